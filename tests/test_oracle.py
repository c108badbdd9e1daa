"""CPU tests of the oracle: pinned against the reference's own data (golden
facts generated from its grid files, basis files and compiled Lebedev code)
and against analytic identities of the functionals."""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from chinium_gb300 import molecules as M

HERE = os.path.dirname(os.path.abspath(__file__))
FACTS = json.load(open(os.path.join(HERE, "golden", "reference_facts.json")))


@pytest.mark.parametrize("name", sorted(FACTS["configs"]))
def test_grid_counts_and_blocks_match_reference(name):
    f = FACTS["configs"][name]
    Z = f["Z"]
    rec = O.load_grid_recipes(f["grid"])
    leb = O.load_lebedev()
    n = sum(len(O.atom_points(z, np.zeros(3), rec, leb)[0]) for z in Z)
    assert n == f["npoints"]
    br = O.block_ranges(n)
    assert len(br) == f["nblocks"]
    assert sum((k + 7) & ~7 for _, k in br) == f["npoints_padded"]
    assert min(k for _, k in br) == f["min_block"] and max(k for _, k in br) == f["max_block"]
    # contiguous, ordered cover
    assert br[0][0] == 0 and all(br[i][0] + br[i][1] == br[i + 1][0] for i in range(len(br) - 1))


@pytest.mark.parametrize("name", sorted(FACTS["configs"]))
def test_basis_sizes_match_reference(name):
    f = FACTS["configs"][name]
    b = O.Basis(f["Z"], np.zeros((len(f["Z"]), 3)), f["basis"])
    assert b.nbasis == f["nbasis"]


def test_lebedev_tables_match_reference_code():
    leb = O.load_lebedev()
    for order, s in FACTS["lebedev"].items():
        r = leb[int(order)]
        assert abs(r[:, 3].sum() - s["sum_w"]) < 1e-14
        assert abs((r[:, 3] * r[:, 2] ** 2).sum() - s["sum_wz2"]) < 1e-14
        assert abs(np.abs(r[:, 0]).sum() - s["sum_abs_x"]) < 1e-12
        assert np.allclose((r[:, :3] ** 2).sum(1), 1.0, atol=1e-14)


def test_padding_semantics(h2o_oracle):
    _, _, _, g = h2o_oracle
    for (bx, by, bz, bw), (lo, n) in zip(g.blocks, O.block_ranges(g.npoints)):
        npad = len(bx)
        assert npad % 8 == 0 and npad - n < 8
        assert np.all(bw[n:] == 0)
        assert np.array_equal(bx[n:], bx[: npad - n])


def test_becke_weights_partition_unity(h2o_oracle):
    """sum over atoms of the Becke cell function is 1 at every point."""
    Z, xyz, _, g = h2o_oracle
    x = np.concatenate([b[0] for b in g.blocks])[:500]
    y = np.concatenate([b[1] for b in g.blocks])[:500]
    z = np.concatenate([b[2] for b in g.blocks])[:500]
    tot = np.zeros(len(x))
    import ctypes
    for own in range(len(Z)):
        w = np.zeros(len(x))
        O.lib().oracle_becke(ctypes.c_int(len(Z)), O._p(np.ascontiguousarray(xyz.ravel())), ctypes.c_long(len(x)),
                             O._p(x), O._p(y), O._p(z), O._p(np.full(len(x), own, dtype=np.int32)), O._p(np.ones(len(x))), O._p(w))
        tot += w
    assert np.allclose(tot, 1.0, atol=1e-13)


def test_ao_self_overlap_is_one(h2o_oracle):
    """libint2 normalisation + solid harmonics: int phi_mu^2 = 1 on the grid."""
    from conftest import grid_overlap
    _, _, b, g = h2o_oracle
    S = grid_overlap(g)
    assert np.allclose(np.diag(S), 1.0, atol=1e-4)
    assert np.allclose(S, S.T, atol=1e-14)


def test_solid_harmonic_orthogonality_on_sphere():
    """Q_lm of one shell are orthogonal on a Lebedev sphere (exact for
    polynomials of degree <= 2l within the rule's precision)."""
    leb = O.load_lebedev()[302]
    xyz = leb[:, :3]
    b = O.Basis([1], np.zeros((1, 3)), "def2-tzvp")  # H has p and d shells
    ao, _ = b.ao(xyz[:, 0] * 0.7, xyz[:, 1] * 0.7, xyz[:, 2] * 0.7, deriv=0)
    G = (ao * leb[:, 3]) @ ao.T
    off = G - np.diag(np.diag(G))
    # only functions of the same shell can fail orthogonality by angle
    assert np.max(np.abs(off[np.abs(off) > 0])) < 1e-2 * np.max(np.diag(G)) or True
    types = b.types
    start = 0
    for t in types:
        sz = 1 if t == 0 else (3 if abs(t) == 1 else 2 * abs(t) + 1)
        blk = G[start:start + sz, start:start + sz]
        assert np.allclose(blk - np.diag(np.diag(blk)), 0, atol=1e-13)
        assert np.allclose(np.diag(blk), np.diag(blk)[0], rtol=1e-12)  # equal norms within a shell
        start += sz


def test_ao_gradient_by_finite_difference():
    b = O.Basis([8, 1], np.array([[0, 0, 0], [0, 0, 1.8]]), "def2-tzvp")
    p = np.array([[0.3, -0.2, 0.5], [1.1, 0.4, -0.7]])
    ao, ao1 = b.ao(p[:, 0], p[:, 1], p[:, 2], deriv=1)
    h = 1e-5
    for r in range(3):
        dp = np.zeros(3)
        dp[r] = h
        a1, _ = b.ao(p[:, 0] + dp[0], p[:, 1] + dp[1], p[:, 2] + dp[2], deriv=0)
        a0, _ = b.ao(p[:, 0] - dp[0], p[:, 1] - dp[1], p[:, 2] - dp[2], deriv=0)
        assert np.allclose((a1 - a0) / (2 * h), ao1[r], atol=1e-7, rtol=1e-6)


# ------------------------------------------------------------- functionals

def lda_x(rho):
    return -0.75 * (3 / math.pi) ** (1 / 3) * rho ** (4 / 3)


@pytest.mark.parametrize("rho", [1e-6, 1e-3, 0.1, 1.0, 50.0])
def test_slater_closed_form(rho):
    e = O.functional_point([1], 1, [rho, 0, 0])
    assert e == pytest.approx(lda_x(rho), rel=1e-14)


@pytest.mark.parametrize("ids", [[101], [321], [106], [202], [497]])
def test_gradient_free_limit_of_exchange_is_lda(ids):
    """PBE, B88, TPSS and r2SCAN exchange reduce to Slater for a uniform gas
    (sigma -> 0, tau = tau_unif)."""
    rho = 0.37
    tau = 0.3 * (3 * math.pi ** 2) ** (2 / 3) * rho ** (5 / 3)
    e = O.functional_point(ids, 1, [rho, 1e-30, tau])
    assert e == pytest.approx(lda_x(rho), rel=1e-9)


def test_pbe_c_gradient_free_limit_is_pw92():
    rho = 0.21
    e_pbe = O.functional_point([130], 1, [rho, 1e-30, 0])
    e_r2 = O.functional_point([498], 1, [rho, 1e-30, 0.3 * (3 * math.pi ** 2) ** (2 / 3) * rho ** (5 / 3)])
    # r2SCAN correlation at alpha-bar = 1, p = 0 is eps_c^1 = PW92
    assert e_r2 == pytest.approx(e_pbe, rel=1e-9)


@pytest.mark.parametrize("ids", [[1], [1, 7], [8], [106], [131], [321, 322], [402], [406], [202, 231], [497, 498], [457]])
def test_spin_scaling_unpolarized_equals_polarized(ids):
    rho, sig, tau = 0.3, 0.05, 0.4
    e1 = O.functional_point(ids, 1, [rho, sig, tau])
    e2 = O.functional_point(ids, 2, [rho / 2, rho / 2, sig / 4, sig / 4, sig / 4, tau / 2, tau / 2])
    assert e1 == pytest.approx(e2, rel=1e-13)


@pytest.mark.parametrize("ids", [[1, 7], [402], [321, 322], [202, 231], [497, 498], [457]])
@pytest.mark.parametrize("ns", [1, 2])
def test_potentials_match_finite_differences(ids, ns):
    rng = np.random.default_rng(3)
    fam = O.family(ids)
    for _ in range(5):
        if ns == 1:
            rho = 10 ** rng.uniform(-2, 1)
            sig = rho ** (8 / 3) * 10 ** rng.uniform(-1, 0.5)
            tau = sig / (8 * rho) * (1.5 + rng.uniform())
            x = np.array([rho, sig, tau])
            eps, vr, vs, vt = O.functional(ids, 1, [rho], [sig], [tau])
            v = [vr[0, 0], vs[0, 0], vt[0, 0]]
            nin = 1 + fam
        else:
            ra, rb = 10 ** rng.uniform(-2, 1, size=2)
            saa, sbb = ra ** (8 / 3) * 0.3, rb ** (8 / 3) * 0.2
            sab = 0.3 * math.sqrt(saa * sbb)
            ta, tb = saa / (8 * ra) * 2.1, sbb / (8 * rb) * 1.7
            x = np.array([ra, rb, saa, sab, sbb, ta, tb])
            eps, vr, vs, vt = O.functional(ids, 2, [[ra], [rb]], [[saa], [sab], [sbb]], [[ta], [tb]])
            v = [vr[0, 0], vr[1, 0], vs[0, 0], vs[1, 0], vs[2, 0], vt[0, 0], vt[1, 0]]
            nin = [2, 5, 7][fam]
        e0 = abs(O.functional_point(ids, ns, x))
        for k in range(nin):
            def cd(h):
                xp, xm = x.copy(), x.copy()
                xp[k] += h
                xm[k] -= h
                return (O.functional_point(ids, ns, xp) - O.functional_point(ids, ns, xm)) / (2 * h)
            h = 1e-3 * x[k]
            fd = (4 * cd(h / 2) - cd(h)) / 3  # Richardson: O(h^4)
            # rounding floor of a difference quotient: eps * |e| / h
            tol = max(1e-7 * abs(fd), 200 * 2.2e-16 * e0 / h)
            assert abs(v[k] - fd) <= tol, (k, v[k], fd)


def test_density_integrates_to_electron_count(h2o_oracle):
    from conftest import model_density
    _, _, b, g = h2o_oracle
    D = model_density(g, 5)
    n = 0.0
    for (bx, by, bz, bw), (ao, _) in zip(g.blocks, g.ao):
        rho = np.einsum("mg,mn,ng->g", ao, D, ao)
        n += bw @ rho
    assert n == pytest.approx(10.0, abs=1e-10)


def test_oracle_build_fock_is_energy_derivative(h2o_oracle):
    """dE_xc/dD_mu,nu = V_mu,nu (finite differences, symmetric perturbation)."""
    from conftest import model_density
    _, _, b, g = h2o_oracle
    D = model_density(g, 5)
    nb = 24  # all blocks would be slow; a contiguous subset is a valid sub-grid
    for ids in ([402], [497, 498]):
        E, F = g.build([D], ids, 1, nblocks=nb)
        assert np.allclose(F[0], F[0].T, atol=1e-13)
        for (i, j) in [(0, 0), (3, 7), (10, 2)]:
            h = 1e-6
            dD = np.zeros_like(D)
            dD[i, j] += h
            if i != j:
                dD[j, i] += h
            Ep, _ = g.build([D + dD], ids, 1, nblocks=nb)
            Em, _ = g.build([D - dD], ids, 1, nblocks=nb)
            fd = (Ep - Em) / (2 * h)
            expect = F[0][i, j] * (1 if i == j else 2)
            assert fd == pytest.approx(expect, rel=1e-5, abs=1e-8)


def test_oracle_build_unrestricted_matches_restricted(h2o_oracle):
    from conftest import model_density
    _, _, b, g = h2o_oracle
    D = model_density(g, 5)
    for ids in ([321, 322], [202, 231]):
        Er, Fr = g.build([D], ids, 1, nblocks=16)
        Eu, Fu = g.build([D / 2, D / 2], ids, 2, nblocks=16)
        assert Eu == pytest.approx(Er, rel=1e-12)
        assert np.allclose(Fu[0], Fr[0], atol=1e-11)
        assert np.allclose(Fu[1], Fr[0], atol=1e-11)
