"""GPU Coulomb and exchange matrices (xc_jk_*, the reference's Int4C2E:
integrals computed on the GPU, contracted with the density matrices) against
the host McMurchie-Davidson repulsion integrals (xc_eri, the full n^4 tensor)
contracted with numpy: J_mn = sum (mn|ls) D_ls, K_mn = sum (ml|ns) D_ls.
Bar: 1e-10 max-abs (the integrals themselves agree to ~1e-14)."""
import ctypes

import numpy as np
import pytest

import chinium_gb300 as cg
from chinium_gb300 import molecules as M
from chinium_gb300._lib import check, lib
from chinium_gb300.scf import JKEngine, repulsion

pytestmark = pytest.mark.gpu

TOL = 1e-10


def sym_density(n, seed, nocc=None):
    rng = np.random.default_rng(seed)
    nocc = nocc or max(1, n // 4)
    A = rng.normal(size=(n, nocc)) * 0.2
    A[np.arange(nocc), np.arange(nocc)] += 1.0
    Q, _ = np.linalg.qr(A)
    return 2 * Q @ Q.T + 0.01 * (lambda B: B + B.T)(rng.normal(size=(n, n)))


CASES = {
    "h2o_svp": (M.h2o, "def2-svp"),
    "h2o_tzvp": (M.h2o, "def2-tzvp"),  # f shells on O
    "water4_svp": (lambda: M.water_clusters(1, seed=5, kmin=4, kmax=4)[0], "def2-svp"),
    # 34 functions: an odd number of function pairs (the dense Coulomb operator's padded row stride)
    "methane_svp": (lambda: M.alkane(1, np.random.default_rng(0)), "def2-svp"),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    mol, name = CASES[request.param]
    Z, xyz = mol()
    b = cg.Basis(Z, xyz, name)
    eri = repulsion(b, threshold=0.0)
    return request.param, b, eri


def reference_jk(eri, D):
    return np.einsum("ijkl,kl->ij", eri, D), np.einsum("ikjl,kl->ij", eri, D)


def test_jk_matches_host_integrals(case):
    name, b, eri = case
    n = b.nbasis
    jk = JKEngine(b, threshold=0.0)
    Ds = [sym_density(n, 1), sym_density(n, 2)]
    Jh, Ks = jk.end(jk.begin(Ds, True))
    J0, K0 = reference_jk(eri, Ds[0])
    J1, K1 = reference_jk(eri, Ds[1])
    dJ = np.abs(Jh - (J0 + J1)).max()
    dK = max(np.abs(Ks[0] - K0).max(), np.abs(Ks[1] - K1).max())
    print("%s: n=%d %s max|dJ| %.2e max|dK| %.2e (max|J| %.2e)" % (name, n, jk.info(), dJ, dK, np.abs(J0).max()))
    assert dJ <= TOL and dK <= TOL
    assert np.allclose(Ks[0], Ks[0].T, atol=1e-13)


def test_direct_mode_equals_incore(case):
    """Integrals recomputed in chunks per build (a memory budget far below
    their size) give the in-core result."""
    name, b, eri = case
    n = b.nbasis
    D = [sym_density(n, 3)]
    a = JKEngine(b, threshold=1e-14)
    c = JKEngine(b, threshold=1e-14, max_bytes=64 * 1024)
    assert a.info()["incore"] and not c.info()["incore"]
    assert a.info()["integrals"] == c.info()["integrals"]
    Ja, Ka = a.end(a.begin(D, True))
    Jc, Kc = c.end(c.begin(D, True))
    assert np.abs(Ja - Jc).max() < 1e-12 and np.abs(Ka[0] - Kc[0]).max() < 1e-12
    # screening at 1e-14 changes nothing at the 1e-10 bar
    Jr, Kr = reference_jk(eri, D[0])
    assert np.abs(Ja - Jr).max() < TOL and np.abs(Ka[0] - Kr).max() < TOL


def test_incore_without_dense_coulomb(case):
    """A budget that holds the integrals but not the dense Coulomb operator
    (the path of large molecules): J and K both from the in-core blocks
    (h2o_tzvp, 28 integrals per quartet: float-float store, exchange summed
    per bra pair in shared memory; the others: FP64 per-quartet kernel);
    equal to the reference and to the dense-operator build, also for J
    alone."""
    name, b, eri = case
    n = b.nbasis
    a = JKEngine(b, threshold=0.0)
    c = JKEngine(b, threshold=0.0, max_bytes=8.0 * a.info()["integrals"])
    assert c.info()["incore"]
    Ds = [sym_density(n, 5), sym_density(n, 6)]
    Jc, Kc = c.end(c.begin(Ds, True))
    Ja, Ka = a.end(a.begin(Ds, True))
    J0, K0 = reference_jk(eri, Ds[0])
    J1, K1 = reference_jk(eri, Ds[1])
    assert np.abs(Jc - (J0 + J1)).max() <= TOL
    assert max(np.abs(Kc[0] - K0).max(), np.abs(Kc[1] - K1).max()) <= TOL
    assert np.abs(Jc - Ja).max() < 1e-12 and np.abs(Kc[1] - Ka[1]).max() < 1e-12
    assert np.abs(c.coulomb(Ds[0]) - J0).max() <= TOL


def test_host_buffer_entry_point(case):
    name, b, eri = case
    n = b.nbasis
    h = ctypes.c_void_p()
    check(lib().xc_jk_create(b._h, 0.0, 0.0, ctypes.byref(h)))
    D = sym_density(n, 4)
    J = np.zeros((n, n))
    check(lib().xc_jk_build(h, 1, D.ctypes.data_as(ctypes.c_void_p), J.ctypes.data_as(ctypes.c_void_p), None))
    lib().xc_jk_destroy(h)
    Jr, _ = reference_jk(eri, D)
    assert np.abs(J - Jr).max() <= TOL
