"""The oracle's response (coupled-perturbed) path on the CPU: second
derivatives of the functionals (order "f") and V_U of getDensityU +
getFockU<u_t>.  The reference ships no golden vectors for these; the oracle is
pinned by closed forms and by V_U being the derivative of the oracle's own
V_xc along D_U (Richardson-extrapolated central differences)."""
import numpy as np
import pytest

from conftest import model_density
from oracle import oracle as O


def test_fxc_slater_closed_form():
    """e = -(3/4)(3/pi)^(1/3) rho^(4/3) (unpolarized); per spin
    e = -(3/4)(6/pi)^(1/3) rho_s^(4/3) with no cross term (polarized)."""
    rho = np.array([1e-6, 0.1, 1.0, 37.0])
    v2 = O.functional_fxc([1], 1, rho)[0][0]
    ana = -(1.0 / 3.0) * (3 / np.pi) ** (1 / 3) * rho ** (-2 / 3)
    assert np.max(np.abs(v2 - ana) / np.abs(ana)) < 1e-11
    r = np.array([[0.3, 0.5, 2.0], [0.2, 0.1, 2.0]])
    v2p = O.functional_fxc([1], 2, r)[0]
    ana_s = -(1.0 / 3.0) * (6 / np.pi) ** (1 / 3) * r ** (-2 / 3)
    assert np.max(np.abs(v2p[0] - ana_s[0]) / np.abs(ana_s[0])) < 1e-11
    assert np.max(np.abs(v2p[2] - ana_s[1]) / np.abs(ana_s[1])) < 1e-11
    assert np.all(v2p[1] == 0)


@pytest.mark.parametrize("ids", [[1, 7], [321, 322], [106, 131], [402]])
def test_fxc_unpolarized_equals_equal_spin_polarized(ids):
    """e(rho, sigma) = e(rho/2, rho/2, sigma/4, sigma/4, sigma/4), so
    v2rho2 = (f_aa + 2 f_ab + f_bb) / 4, v2rhosigma = sum_(s,x) f_(rho_s sigma_x) / 8
    and v2sigma2 = sum_(x,y) f_(sigma_x sigma_y) / 16: the unpolarized and the
    polarized code paths of the oracle agree (sigma_ab sits on its clamp here,
    so the polarized side also exercises the one-sided steps, good to ~1e-9
    per entry; the sums cancel entries of opposite sign, hence 2e-7)."""
    rho = np.array([0.02, 0.3, 1.5])
    sig = np.array([0.001, 0.05, 0.9])
    u = O.functional_fxc(ids, 1, rho, sig)
    p = O.functional_fxc(ids, 2, np.stack([rho / 2, rho / 2]), np.stack([sig / 4] * 3))
    assert np.allclose(u[0][0], (p[0][0] + 2 * p[0][1] + p[0][2]) / 4, rtol=2e-7, atol=0)
    if O.family(ids) >= 1:
        assert np.allclose(u[1][0], p[1].sum(0) / 8, rtol=2e-7, atol=0)
        f = p[2]
        tot = f[0] + f[3] + f[5] + 2 * (f[1] + f[2] + f[4])
        assert np.allclose(u[2][0], tot / 16, rtol=2e-7, atol=0)


def test_fxc_rejects_meta_gga():
    with pytest.raises(ValueError):
        O.functional_fxc([202, 231], 1, np.array([0.1]), np.array([0.01]))


def _dv_fd(og, D, U, ids, nspin, h=5e-5):
    def V(Dx):
        return np.array(og.build(Dx, ids, nspin)[1])

    def cd(hh):
        return (V(D + hh * U) - V(D - hh * U)) / (2 * hh)

    return (4 * cd(h / 2) - cd(h)) / 3


@pytest.mark.parametrize("name,nspin", [("SVWN5", 1), ("PBE", 1), ("B3LYP", 1), ("PBE", 2), ("BLYP", 2)])
def test_oracle_response_is_derivative_of_fock(h2o_oracle, name, nspin):
    """V_U(D_U) = d V_xc(D + e D_U) / de at e = 0 (restricted: the reference's
    expression; unrestricted: libxc's layouts with S on the output pair)."""
    Z, xyz, basis, og = h2o_oracle
    n = basis.nbasis
    ids = O.FUNCTIONAL_FILES[name]
    D = model_density(og, 5)[None] if nspin == 1 else np.stack(model_density(og, (5, 4), nspin=2, seed=2))
    rng = np.random.default_rng(7)
    U = rng.normal(size=(nspin, 2, n, n)) * 0.05
    U = U + U.transpose(0, 1, 3, 2)
    FU = og.response(D, U, ids, nspin)
    for m in range(2):
        ref = _dv_fd(og, D, U[:, m], ids, nspin)
        err = np.abs(FU[:, m] - ref).max()
        assert err < 5e-10, (name, nspin, m, err, np.abs(ref).max())
    # V_U is linear in D_U and symmetric
    FU2 = og.response(D, U[:, :1] * 3.0, ids, nspin)
    assert np.allclose(FU2[:, 0], 3.0 * FU[:, 0], rtol=0, atol=1e-13)
    assert np.allclose(FU, FU.transpose(0, 1, 3, 2), rtol=0, atol=1e-14)


def test_oracle_response_nonsymmetric_orientation(h2o_oracle):
    """For a non-symmetric D_U the gradient term uses 2 sum D_U(mu, nu)
    grad phi_mu phi_nu (GridDensity.cpp:67-68): V_U(D_U) differs from V_U(D_U^T)
    by the antisymmetric part's gradient contribution, and the symmetric part
    alone gives the average."""
    Z, xyz, basis, og = h2o_oracle
    n = basis.nbasis
    ids = O.FUNCTIONAL_FILES["PBE"]
    D = model_density(og, 5)[None]
    rng = np.random.default_rng(11)
    A = rng.normal(size=(n, n)) * 0.05
    U = np.stack([A, A.T, 0.5 * (A + A.T)])[None]
    FU = og.response(D, U, ids, 1)
    assert np.abs(FU[0, 0] - FU[0, 1]).max() > 1e-6
    assert np.allclose(0.5 * (FU[0, 0] + FU[0, 1]), FU[0, 2], rtol=0, atol=1e-13)


@pytest.mark.parametrize("name", ["SVWN5", "PBE", "BLYP"])
def test_oracle_unrestricted_response_at_equal_spins_is_restricted(h2o_oracle, name):
    """With D_a = D_b = D / 2 and D_U,a = D_U,b = D_U / 2 each spin's V_U is the
    restricted V_U of (D, D_U): the unrestricted expression (libxc layouts, the
    S = 2 factor on the output sigma pair) is the derivative of V_xc at a
    closed shell too.  sigma_ab sits on its clamp there, so the oracle's
    one-sided steps carry the check (~1e-9)."""
    Z, xyz, basis, og = h2o_oracle
    n = basis.nbasis
    ids = O.FUNCTIONAL_FILES[name]
    D = model_density(og, 5)
    rng = np.random.default_rng(13)
    A = rng.normal(size=(n, n)) * 0.05
    U = A + A.T
    r = og.response(D[None], U[None, None], ids, 1)[0, 0]
    u = og.response(np.stack([D / 2, D / 2]), np.stack([U / 2, U / 2])[:, None], ids, 2)
    scale = np.abs(r).max()
    for s in range(2):
        assert np.abs(u[s, 0] - r).max() < 1e-8 * scale, (name, s, np.abs(u[s, 0] - r).max())


@pytest.mark.parametrize("name,nspin", [("PBE", 1), ("SVWN5", 2)])
def test_parallel_response_driver_equals_block_loop(h2o_oracle, name, nspin):
    """The OpenMP response driver (the timed CPU baseline) gives the per-block restatement's V_U."""
    Z, xyz, basis, og = h2o_oracle
    n = basis.nbasis
    ids = O.FUNCTIONAL_FILES[name]
    D = model_density(og, 5)[None] if nspin == 1 else np.stack(model_density(og, (5, 4), nspin=2, seed=2))
    rng = np.random.default_rng(3)
    U = rng.normal(size=(nspin, 2, n, n)) * 0.05
    U = U + U.transpose(0, 1, 3, 2)
    a = og.response(D, U, ids, nspin)
    b = og.build_response(D, U, ids, nspin, nthreads=4)
    assert np.abs(a - b).max() < 1e-13
