"""GPU parity of the response (coupled-perturbed) path through the C ABI:
second derivatives of the functionals (Evaluate("f")) against the oracle's
complex-step + Richardson values, and V_U of getDensityU + getFockU<u_t>
against the oracle's restatement and against central differences of the
CUDA FP64 V_xc.  Tolerances: V_U 1e-10 max-abs against the oracle (the FP64
parity bar); f_xc relative 1e-9 for v2rho2, 1e-8 for v2rhosigma and 5e-8
for v2sigma2, the accuracy of the oracle's differences of complex-step
derivatives (v_sigma moves with sigma only at order s^2 for small reduced
gradients s, which costs v2sigma2 digits there; the CUDA jets are exact
derivatives of the same expressions)."""
import numpy as np
import pytest

import chinium_gb300 as cg
from chinium_gb300 import molecules as M
from conftest import model_density
from oracle import oracle as O

pytestmark = pytest.mark.gpu

V_TOL = 1e-10
FXC_RTOL = (1e-9, 1e-8, 5e-8)  # v2rho2, v2rhosigma, v2sigma2


@pytest.fixture(scope="module")
def h2o(h2o_oracle):
    Z, xyz, ob, og = h2o_oracle
    b = cg.Basis(Z, xyz, "def2-svp")
    return Z, xyz, b, ob, og


def random_points(nspin, n, seed):
    """Densities 1e-4..10, reduced gradients s = |grad rho| / rho^(4/3) in
    0.05..3, spin densities within a factor 10 of each other and sigma_ab at
    0.1..0.9 of its Cauchy-Schwarz bound, plus three points at or below the
    1e-15 threshold.  Outside this range (s -> 0, one spin vanishing, sigma_ab
    -> 0) the oracle's finite differences of its complex-step derivatives lose
    digits (v_sigma hardly moves with sigma; rounding of 1 +- zeta), while the
    CUDA jets stay exact: the grid tests cover those points through V_U."""
    rng = np.random.default_rng(seed)
    if nspin == 1:
        rho = 10.0 ** rng.uniform(-4, 1, n)
        rho[:3] = [1e-17, 0.0, 2e-16]
        sig = (rng.uniform(0.05, 3, n) * rho ** (4 / 3)) ** 2
        return rho[None], sig[None]
    ra = 10.0 ** rng.uniform(-4, 1, n)
    rb = ra * 10.0 ** rng.uniform(-1, 1, n)
    rho = np.stack([ra, rb])
    rho[:, :3] = [[1e-17, 0.0, 4e-16], [1e-17, 0.0, 5e-16]]
    ga = rng.uniform(0.05, 3, n) * rho[0] ** (4 / 3)
    gb = rng.uniform(0.05, 3, n) * rho[1] ** (4 / 3)
    c = rng.uniform(0.1, 0.9, n) * rng.choice([-1.0, 1.0], n)
    return rho, np.stack([ga * ga, c * ga * gb, gb * gb])


def close(a, b, rtol):
    scale = np.abs(b).max() if b.size else 0.0
    return np.all(np.abs(a - b) <= rtol * np.abs(b) + 1e-13 * scale)


@pytest.mark.parametrize("name", ["SLATER", "SVWN5", "PBE", "BLYP", "B3LYP", "PBE0", "BHHLYP"])
@pytest.mark.parametrize("nspin", [1, 2])
def test_fxc_points_match_oracle(name, nspin):
    ids = O.FUNCTIONAL_FILES[name]
    rho, sig = random_points(nspin, 256, seed=5 + nspin)
    xc = cg.ExchangeCorrelation(spin=nspin).Read(name)
    got = xc.fxc_points(rho, sig)
    ref = O.functional_fxc(ids, nspin, rho, sig)
    fam = O.family(ids)
    for k, (a, b) in enumerate(zip(got, ref)):
        if fam == 0 and k > 0:
            continue
        assert close(a, b, FXC_RTOL[k]), (name, nspin, k, np.abs(a - b).max(), np.abs(b).max())
    # below the density threshold every second derivative is zero
    for a in got:
        assert np.all(a[:, :3] == 0)


def test_fxc_rejects_meta_gga():
    xc = cg.ExchangeCorrelation().Read("TPSS")
    with pytest.raises(cg.XCError) as e:
        xc.fxc_points(np.array([[0.1]]), np.array([[0.01]]))
    assert e.value.code == -6


def response_case(og, n, nspin, seed=7):
    D = [model_density(og, 5)] if nspin == 1 else model_density(og, (5, 4), nspin=2, seed=2)
    rng = np.random.default_rng(seed)
    U = rng.normal(size=(nspin, 3, n, n)) * 0.05
    U[:, :2] = U[:, :2] + U[:, :2].transpose(0, 1, 3, 2)  # two symmetric, one general matrix
    return D, U


@pytest.mark.parametrize("name,nspin", [("SLATER", 1), ("SVWN5", 1), ("PBE", 1), ("B3LYP", 1),
                                        ("SVWN5", 2), ("PBE", 2), ("BLYP", 2)])
def test_response_fock_matches_oracle(h2o, name, nspin):
    """build_response (getDensity + Evaluate("ev", "f") + getDensityU +
    getFockU<u_t>) against the oracle, including a non-symmetric D_U."""
    Z, xyz, b, ob, og = h2o
    n = b.nbasis
    ids = O.FUNCTIONAL_FILES[name]
    fam = O.family(ids)
    D, U = response_case(og, n, nspin)
    g = cg.Grid(b, "SG-1", nspin=nspin)
    g.setType(fam)
    g.getAO(0)
    xc = cg.ExchangeCorrelation(spin=nspin).Read(name)
    FU = np.array(g.build_response(xc, D, [list(U[s]) for s in range(nspin)]))
    ref = og.response(np.stack(D), U, ids, nspin)
    err = np.abs(FU - ref).max()
    print(name, nspin, "max |dV_U| %.2e, max |V_U| %.2e" % (err, np.abs(ref).max()))
    assert err < V_TOL


def test_response_split_calls_equal_fused(h2o):
    """Evaluate("f") + getDensityU + getFockU<u_t> after getDensity +
    Evaluate("ev") give the fused call's matrices; call-order errors are
    reported as XC_ERR_STATE."""
    Z, xyz, b, ob, og = h2o
    n = b.nbasis
    D, U = response_case(og, n, 1)
    xc = cg.ExchangeCorrelation().Read("PBE")
    g = cg.Grid(b, "SG-1")
    g.setType(1)
    g.getAO(0)
    fused = np.array(g.build_response(xc, D, list(U[0])))
    g2 = cg.Grid(b, "SG-1")
    g2.setType(1)
    g2.getAO(0)
    g2.getDensity(D)
    with pytest.raises(cg.XCError) as e:  # no Evaluate("f") yet
        g2.getDensityU(list(U[0]))
        g2.getFockU()
    assert e.value.code == -4
    xc.Evaluate("ev", g2)
    xc.Evaluate("f", g2)
    g2.getDensityU(list(U[0]))
    split = np.array(g2.getFockU())
    assert np.abs(split - fused).max() < 1e-13
    # a new density invalidates the second derivatives
    g2.getDensity(D)
    with pytest.raises(cg.XCError) as e:
        g2.getFockU()
    assert e.value.code == -4


def test_response_rejects_meta_gga(h2o):
    Z, xyz, b, ob, og = h2o
    D, U = response_case(og, b.nbasis, 1)
    xc = cg.ExchangeCorrelation().Read("TPSS")
    g = cg.Grid(b, "SG-1")
    g.setType(2)
    g.getAO(0)
    with pytest.raises(cg.XCError) as e:
        g.build_response(xc, D, list(U[0]))
    assert e.value.code == -6


def bench_density(nbasis, nocc, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(nbasis, nocc)) * 0.05
    A[np.arange(nocc), np.arange(nocc)] += 1.0
    Q, _ = np.linalg.qr(A)
    return 2.0 * Q @ Q.T


@pytest.mark.parametrize("case", ["c18", "fe4s4"])
def test_response_is_derivative_of_gpu_fock(case):
    """Size-independent property at a production size: V_U(D_U) equals the
    Richardson-extrapolated central difference of the CUDA FP64 V_xc along
    D_U (C18 B3LYP/def2-TZVP SG-2 RKS; Fe4S4 PBE/def2-SVP SG-2 UKS), on
    screened grids (the response uses the same blocks as V_xc)."""
    if case == "c18":
        Z, xyz = M.c18()
        b = cg.Basis(Z, xyz, "def2-tzvp")
        name, nspin, grid = "B3LYP", 1, "SG-2"
        D = [bench_density(b.nbasis, 54)]
    else:
        Z, xyz = M.fe4s4()
        b = cg.Basis(Z, xyz, "def2-svp")
        name, nspin, grid = "PBE", 2, "SG-2"
        ne = sum(Z)
        D = [0.5 * bench_density(b.nbasis, (ne + 8) // 2, 1), 0.5 * bench_density(b.nbasis, (ne - 8) // 2, 2)]
    n = b.nbasis
    g = cg.Grid(b, grid, nspin=nspin, screen_threshold=1e-11)
    g.setType(1)
    g.getAO(0)
    xc = cg.ExchangeCorrelation(spin=nspin).Read(name)
    rng = np.random.default_rng(3)
    U = rng.normal(size=(nspin, n, n)) * 0.01
    U = U + U.transpose(0, 2, 1)
    FU = np.array(g.build_response(xc, D, [[U[s]] for s in range(nspin)]))[:, 0]

    def V(h):
        return np.array(g.build(xc, [D[s] + h * U[s] for s in range(nspin)])[1])

    def cd(h):
        return (V(h) - V(-h)) / (2 * h)

    h = 5e-5
    ref = (4 * cd(h / 2) - cd(h)) / 3
    err = np.abs(FU - ref).max()
    print(case, "max |dV_U| %.2e, max |V_U| %.2e" % (err, np.abs(ref).max()))
    assert err < 1e-8 * max(1.0, np.abs(ref).max())


MIXED_RTOL = 5e-6  # of max |V_U|: split-BF16 products with FP32 accumulation per unit, FP64 sums


@pytest.mark.parametrize("name,nspin", [("SVWN5", 1), ("PBE", 1), ("B3LYP", 1), ("PBE", 2)])
def test_response_mixed_matches_fp64(h2o, name, nspin):
    """Tensor-core response densities and V_U (FP64 ground state) against the
    FP64 response on symmetric D_U; a non-symmetric D_U gives exactly the
    result of its symmetric part."""
    Z, xyz, b, ob, og = h2o
    n = b.nbasis
    fam = O.family(O.FUNCTIONAL_FILES[name])
    D, U = response_case(og, n, nspin)
    g = cg.Grid(b, "SG-1", nspin=nspin)
    g.setType(fam)
    g.getAO(0)
    xc = cg.ExchangeCorrelation(spin=nspin).Read(name)
    Us = [list(U[s, :2]) for s in range(nspin)]
    ref = np.array(g.build_response(xc, D, Us))
    got = np.array(g.build_response(xc, D, Us, precision=cg.PRECISION_MIXED))
    err = np.abs(got - ref).max()
    print(name, nspin, "mixed max |dV_U| %.2e, max |V_U| %.2e" % (err, np.abs(ref).max()))
    assert err < MIXED_RTOL * np.abs(ref).max()
    A = U[:, 2]
    sym = 0.5 * (A + A.transpose(0, 2, 1))
    ga = np.array(g.build_response(xc, D, [[A[s]] for s in range(nspin)], precision=cg.PRECISION_MIXED))
    gs = np.array(g.build_response(xc, D, [[sym[s]] for s in range(nspin)], precision=cg.PRECISION_MIXED))
    assert np.array_equal(ga, gs)


def test_response_mixed_c18_b3lyp():
    """C18 B3LYP/def2-TZVP SG-2: the tensor-core response of three symmetric
    perturbations against the FP64 response (screened grid)."""
    Z, xyz = M.c18()
    b = cg.Basis(Z, xyz, "def2-tzvp")
    n = b.nbasis
    g = cg.Grid(b, "SG-2", screen_threshold=1e-11)
    g.setType(1)
    g.getAO(0)
    xc = cg.ExchangeCorrelation().Read("B3LYP")
    D = [bench_density(n, 54)]
    rng = np.random.default_rng(5)
    A = rng.normal(size=(3, n, n)) * 0.01
    U = [list(A + A.transpose(0, 2, 1))]
    ref = np.array(g.build_response(xc, D, U))
    got = np.array(g.build_response(xc, D, U, precision=cg.PRECISION_MIXED))
    err = np.abs(got - ref).max()
    print("c18 mixed max |dV_U| %.2e, max |V_U| %.2e" % (err, np.abs(ref).max()))
    assert err < MIXED_RTOL * np.abs(ref).max()


def test_response_mixed_split_calls_equal_fused(h2o):
    """setResponsePrecision(MIXED) + getDensityU + getFockU on the ground state
    of getDensity + Evaluate("ev", "f") give the fused mixed call's matrices;
    a second iteration reuses the tile-order ground state."""
    Z, xyz, b, ob, og = h2o
    D, U = response_case(og, b.nbasis, 1)
    xc = cg.ExchangeCorrelation().Read("PBE")
    g = cg.Grid(b, "SG-1")
    g.setType(1)
    g.getAO(0)
    Us = list(U[0, :2])
    fused = np.array(g.build_response(xc, D, Us, precision=cg.PRECISION_MIXED))
    g.getDensity(D)
    xc.Evaluate("ev", g)
    xc.Evaluate("f", g)
    g.setResponsePrecision(cg.PRECISION_MIXED)
    for _ in range(2):
        g.getDensityU(Us)
        split = np.array(g.getFockU())
        assert np.array_equal(split, fused)
    g.setResponsePrecision(cg.PRECISION_FP64)
    g.getDensityU(Us)
    f64 = np.array(g.getFockU())
    assert np.abs(f64 - split).max() < MIXED_RTOL * np.abs(f64).max()


@pytest.mark.parametrize("name", ["PBE", "B3LYP"])
def test_unrestricted_response_at_equal_spins_is_restricted(h2o, name):
    """CUDA FP64: D_a = D_b = D / 2, D_U,a = D_U,b = D_U / 2 give each spin the
    restricted V_U of (D, D_U) (sigma_ab on its clamp: the jets keep the
    unclamped branch, as the first derivatives do)."""
    Z, xyz, b, ob, og = h2o
    n = b.nbasis
    D = model_density(og, 5)
    rng = np.random.default_rng(17)
    A = rng.normal(size=(n, n)) * 0.05
    U = A + A.T
    gr = cg.Grid(b, "SG-1")
    gr.setType(1)
    gr.getAO(0)
    r = np.array(gr.build_response(cg.ExchangeCorrelation().Read(name), [D], [U]))[0, 0]
    gu = cg.Grid(b, "SG-1", nspin=2)
    gu.setType(1)
    gu.getAO(0)
    u = np.array(gu.build_response(cg.ExchangeCorrelation(spin=2).Read(name), [D / 2, D / 2], [[U / 2], [U / 2]]))
    for s in range(2):
        assert np.abs(u[s, 0] - r).max() < 1e-12 * max(1.0, np.abs(r).max())


@pytest.mark.parametrize("name,nspin", [("SVWN5", 1), ("PBE", 1), ("PBE", 2)])
def test_hessian_skeleton_fock_terms_match_oracle(h2o, name, nspin):
    """getFockSkeleton and getFockU<s_t> (grid fixed, FP64) against the oracle's
    restatement, whose sum the CPU tests pin to finite differences of V_xc."""
    Z, xyz, b, ob, og = h2o
    ids = O.FUNCTIONAL_FILES[name]
    fam = O.family(ids)
    D = [model_density(og, 5)] if nspin == 1 else model_density(og, (5, 4), nspin=2, seed=2)
    g = cg.Grid(b, "SG-1", nspin=nspin)
    g.setType(fam)
    g.getAO(1)
    xc = cg.ExchangeCorrelation(spin=nspin).Read(name)
    FS, FU = g.getFockSkeleton(xc, D)
    rs, ru = og.fock_skeleton(np.stack(D), ids, nspin)
    es, eu = np.abs(FS - rs).max(), np.abs(FU - ru).max()
    print(name, nspin, "skeleton max |dF| %.2e (max %.2e), s_t response %.2e (max %.2e)"
          % (es, np.abs(rs).max(), eu, np.abs(ru).max()))
    assert es < V_TOL and eu < V_TOL
