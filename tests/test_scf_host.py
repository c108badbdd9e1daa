"""Host-side pieces of the SCF caller (no GPU): the DIIS extrapolation with
its kept inner products against a from-scratch restatement of Pulay's
commutator DIIS (src/DIIS/CDIIS.cpp:24-47), and the packed-pair Coulomb
contraction used by the HBM-resident J."""
import numpy as np

from chinium_gb300.scf import DIIS, coulomb_from_pairs, coulomb_pairs


def _pulay(Fs, Es):
    m = len(Fs)
    B = -np.ones((m + 1, m + 1))
    B[m, m] = 0
    for i in range(m):
        for j in range(m):
            B[i, j] = sum(np.vdot(a, b) for a, b in zip(Es[i], Es[j]))
    rhs = np.zeros(m + 1)
    rhs[m] = -1
    c = np.linalg.solve(B + np.eye(m + 1) * 1e-14 * np.abs(B).max() * (np.arange(m + 1) < m), rhs)[:m]
    return [sum(ci * F[s] for ci, F in zip(c, Fs)) for s in range(len(Fs[0]))]


def test_diis_kept_products_match_full_recompute():
    rng = np.random.default_rng(7)
    d = DIIS(size=5)
    Fs, Es = [], []
    for it in range(9):
        F = [rng.normal(size=(6, 6)) for _ in range(2)]
        E = [rng.normal(size=(6, 6)) * 0.5 ** it for _ in range(2)]
        d.push(F, E)
        Fs.append(F)
        Es.append(E)
        Fs, Es = Fs[-5:], Es[-5:]
        got = d.extrapolate()
        if len(Fs) < 2:
            continue
        want = _pulay(Fs, Es)
        for a, b in zip(got, want):
            np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12)


def test_packed_pair_coulomb_matches_full_contraction():
    """J_mn = sum_ls (mn|ls) D_ls through the (n(n+1)/2)^2 pair matrix and
    the packed density with doubled off-diagonal elements."""
    rng = np.random.default_rng(3)
    n = 7
    A = rng.normal(size=(n, n, n, n))
    eri = A + A.transpose(1, 0, 2, 3)
    eri = eri + eri.transpose(0, 1, 3, 2)
    eri = eri + eri.transpose(2, 3, 0, 1)
    D = rng.normal(size=(n, n))
    D = D + D.T
    P, iu, ju, w = coulomb_pairs(eri)
    assert P.shape == (n * (n + 1) // 2,) * 2
    J = coulomb_from_pairs(P @ (D[iu, ju] * w), iu, ju, n)
    np.testing.assert_allclose(J, np.einsum("mnls,ls->mn", eri, D), rtol=1e-12, atol=1e-12)
