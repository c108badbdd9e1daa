"""Host-side pieces of the SCF caller (no GPU): the DIIS extrapolation with
its kept inner products against a from-scratch restatement of Pulay's
commutator DIIS (src/DIIS/CDIIS.cpp:24-47), and the packed-pair Coulomb
contraction used by the HBM-resident J."""
import numpy as np
import pytest

from chinium_gb300.scf import DIIS


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


def test_canonical_quartet_jk_algebra_matches_full_contraction():
    """The contraction rule of the GPU J/K engine (k_eri.cu), restated: every
    unique shell quartet (a >= b, c >= d, bra pair >= ket pair, pairs in any
    order) contributes its full function block once, scaled by 1/2 for each
    of a == b, c == d and equal pairs, to rawJ(a,b), rawJ(c,d), rawK(a,c),
    rawK(b,d), rawK(a,d), rawK(b,c); then J = 2 (rawJ + rawJ^T) and
    K = rawK + rawK^T are the full contractions J_mn = sum (mn|ls) D_ls and
    K_mn = sum (ml|ns) D_ls."""
    rng = np.random.default_rng(3)
    sizes = [1, 3, 1, 5, 3, 7]
    first = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    n = sum(sizes)
    A = rng.normal(size=(n, n, n, n))
    eri = A + A.transpose(1, 0, 2, 3)
    eri = eri + eri.transpose(0, 1, 3, 2)
    eri = eri + eri.transpose(2, 3, 0, 1)
    D = rng.normal(size=(n, n))
    D = D + D.T
    pairs = [(a, b) for a in range(len(sizes)) for b in range(a + 1)]
    rng.shuffle(pairs)  # the engine orders pairs by their Schwarz bound: any order works
    rawJ, rawK = np.zeros((n, n)), np.zeros((n, n))
    sl = lambda s: slice(first[s], first[s] + sizes[s])
    for i, (a, b) in enumerate(pairs):
        for j in range(i + 1):
            c, d = pairs[j]
            f = (0.5 if a == b else 1.0) * (0.5 if c == d else 1.0) * (0.5 if i == j else 1.0)
            I = f * eri[sl(a), sl(b), sl(c), sl(d)]
            rawJ[sl(a), sl(b)] += np.einsum("abcd,cd->ab", I, D[sl(c), sl(d)])
            rawJ[sl(c), sl(d)] += np.einsum("abcd,ab->cd", I, D[sl(a), sl(b)])
            rawK[sl(a), sl(c)] += np.einsum("abcd,bd->ac", I, D[sl(b), sl(d)])
            rawK[sl(b), sl(d)] += np.einsum("abcd,ac->bd", I, D[sl(a), sl(c)])
            rawK[sl(a), sl(d)] += np.einsum("abcd,bc->ad", I, D[sl(b), sl(c)])
            rawK[sl(b), sl(c)] += np.einsum("abcd,ad->bc", I, D[sl(a), sl(d)])
    J = 2 * (rawJ + rawJ.T)
    K = rawK + rawK.T
    np.testing.assert_allclose(J, np.einsum("mnls,ls->mn", eri, D), rtol=1e-12, atol=1e-11)
    np.testing.assert_allclose(K, np.einsum("mlns,ls->mn", eri, D), rtol=1e-12, atol=1e-11)


def test_adiis_start_and_cayley_rotations_reach_the_diagonalisation_fixed_point(monkeypatch):
    """Restricted Hartree-Fock on the host (XC switched off, host integrals):
    the SCF with the reference's ADIIS start (until the commutator is below
    1e-1) and Cayley rotations of the orbitals in place of diagonalisations
    (below 1e-2) converges to the energy and density of plain CDIIS with a
    full diagonalisation every iteration."""
    import chinium_gb300 as cg
    from chinium_gb300 import molecules as M
    from chinium_gb300 import scf

    class NoXC:
        EXX = 1.0  # Hartree-Fock exchange
        type = 0

        def __init__(self, spin=1):
            pass

        def Read(self, name):
            return self

    class NoXCGrid:
        def __init__(self, n):
            self.n = n

        def build(self, xc, D, precision=0):
            return 0.0, [np.zeros((self.n, self.n)) for _ in D]

    monkeypatch.setattr(scf, "ExchangeCorrelation", NoXC)
    Z, xyz = M.h2o()
    b = cg.Basis(Z, xyz, "def2-svp")
    S, T, V = scf.one_electron(b)
    out = {}
    for name, kw in (("plain", dict(adiis_until=0.0, rotate_below=0.0)), ("adiis_cayley", {})):
        ctx = {"basis": b, "S": S, "H": T + V, "jk": scf.JK(scf.repulsion(b, 0.0)), "grid": NoXCGrid(b.nbasis),
               "Enuc": M.nuclear_repulsion(Z, xyz), "grid_key": ("grid", 1, "HF", "SG-1", 0.0)}
        r = scf.run_scf(Z, xyz, functional="HF", guess="core", context=ctx, conv_energy=1e-10, jk_device="cpu", **kw)
        assert r.converged
        out[name] = r
    assert out["adiis_cayley"].timings.get("rotations", 0) > 0
    assert abs(out["plain"].energy - out["adiis_cayley"].energy) < 1e-9
    assert np.abs(out["plain"].D[0] - out["adiis_cayley"].D[0]).max() < 1e-5
    assert -76.1 < out["plain"].energy < -75.8  # RHF / def2-SVP water


def test_cayley_closed_form_matches_the_explicit_transform():
    """cayley_update's occupied-block closed form equals C (1 - K/2)^-1 (1 + K/2)
    built explicitly, and keeps the orbitals S-orthonormal."""
    from chinium_gb300.scf import cayley_update
    rng = np.random.default_rng(3)
    n, nocc = 30, 7
    A = rng.normal(size=(n, n))
    S = A @ A.T / n + np.eye(n)
    w, Q = np.linalg.eigh(S)
    X = Q @ np.diag(w ** -0.5) @ Q.T  # S^-1/2
    F0 = np.diag(np.sort(rng.normal(size=n)) * 3)  # well-separated orbital energies
    C = X @ np.linalg.qr(rng.normal(size=(n, n)))[0]
    F = np.linalg.inv(C.T) @ F0 @ np.linalg.inv(C)  # C^T F C = F0
    P = rng.normal(size=(n, n)) * 0.02
    F = F + P + P.T  # occupied-virtual coupling
    got = cayley_update(C, F, nocc)
    Fm = C.T @ F @ C
    e = np.diag(Fm)
    o, v = slice(0, nocc), slice(nocc, n)
    kap = -Fm[v, o] / (e[v][:, None] - e[o][None, :])
    K = np.zeros((n, n))
    K[v, o] = kap
    K[o, v] = -kap.T
    want = C @ np.linalg.solve(np.eye(n) - 0.5 * K, np.eye(n) + 0.5 * K)
    np.testing.assert_allclose(got, want, atol=1e-12)
    np.testing.assert_allclose(got.T @ S @ got, np.eye(n), atol=1e-11)


def _host_hf(monkeypatch, Z, xyz, basis, mult):
    """Hartree-Fock through run_scf with the XC build switched off and the
    host integrals (as in the test above)."""
    import chinium_gb300 as cg
    from chinium_gb300 import molecules as M
    from chinium_gb300 import scf

    class NoXC:
        EXX = 1.0
        type = 0

        def __init__(self, spin=1):
            pass

        def Read(self, name):
            return self

    class NoXCGrid:
        def __init__(self, n):
            self.n = n

        def build(self, xc, D, precision=0):
            return 0.0, [np.zeros((self.n, self.n)) for _ in D]

    monkeypatch.setattr(scf, "ExchangeCorrelation", NoXC)
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    b = cg.Basis(Z, xyz, basis)
    S, T, V = scf.one_electron(b)
    nspin = 2 if mult != 1 else 1
    ctx = {"basis": b, "S": S, "H": T + V, "jk": scf.JK(scf.repulsion(b, 0.0)), "grid": NoXCGrid(b.nbasis),
           "Enuc": M.nuclear_repulsion(Z, xyz), "grid_key": ("grid", nspin, "HF", "SG-1", 0.0)}
    r = scf.run_scf(Z, xyz, basis=basis, functional="HF", mult=mult, guess="core", context=ctx,
                    conv_energy=1e-11, jk_device="cpu")
    assert r.converged
    return r, S, T + V


def test_one_electron_hartree_fock_is_the_core_eigenvalue(monkeypatch):
    """For one electron, Coulomb and exchange cancel exactly (J = K of the
    same spin density), so the UHF energy of the hydrogen atom is the lowest
    eigenvalue of the core Hamiltonian in the basis: a check of the host
    integrals' J / K, the unrestricted Fock assembly and the energy
    expression; variationally above the exact -1/2 Eh."""
    import scipy.linalg as sl
    for basis in ("def2-svp", "def2-tzvp"):
        r, S, H = _host_hf(monkeypatch, [1], [0.0, 0.0, 0.0], basis, mult=2)
        e0 = sl.eigh(H, S, eigvals_only=True)[0]
        assert abs(r.energy - e0) < 1e-10, (basis, r.energy, e0)
        assert -0.5 < r.energy < -0.499


def test_helium_hartree_fock_above_the_limit(monkeypatch):
    """RHF of the helium atom: variationally above the numerical Hartree-Fock
    limit, -2.8616800 Eh, and within 2 mEh of it in def2-TZVP, whose helium
    set is 3s1p (the integrals, J - K / 2 of a two-electron closed shell and
    the SCF together; a wrong sign or scale of J or K moves it by ~1 Eh)."""
    r, _, _ = _host_hf(monkeypatch, [2], [0.0, 0.0, 0.0], "def2-tzvp", mult=1)
    assert -2.8616800 < r.energy < -2.8596800, r.energy


def test_unrestricted_adiis_and_rotations_reach_the_diagonalisation_fixed_point(monkeypatch):
    """UHF of the OH radical (doublet; both spin channels occupied, unequal):
    the ADIIS start and Cayley rotations per spin reach the energy of plain
    CDIIS with a diagonalisation every iteration."""
    r_rot, _, _ = _host_hf(monkeypatch, [8, 1], [0, 0, 0, 0, 0, 1.83], "def2-svp", mult=2)  # defaults
    import chinium_gb300 as cg
    from chinium_gb300 import molecules as M
    from chinium_gb300 import scf
    Z, xyz = [8, 1], np.array([[0, 0, 0], [0, 0, 1.83]], dtype=np.float64)
    b = cg.Basis(Z, xyz, "def2-svp")
    S, T, V = scf.one_electron(b)

    class NoXCGrid:
        def build(self, xc, D, precision=0):
            return 0.0, [np.zeros((b.nbasis, b.nbasis)) for _ in D]

    ctx = {"basis": b, "S": S, "H": T + V, "jk": scf.JK(scf.repulsion(b, 0.0)), "grid": NoXCGrid(),
           "Enuc": M.nuclear_repulsion(Z, xyz), "grid_key": ("grid", 2, "HF", "SG-1", 0.0)}
    r_plain = scf.run_scf(Z, xyz, basis="def2-svp", functional="HF", mult=2, guess="core", context=ctx,
                          conv_energy=1e-10, jk_device="cpu", adiis_until=0.0, rotate_below=0.0)
    assert r_plain.converged and r_plain.timings.get("rotations", 0) == 0
    assert r_rot.timings.get("rotations", 0) > 0
    assert abs(r_rot.energy - r_plain.energy) < 1e-9
    assert -75.2 < r_rot.energy < -75.1


def _hf_atom(monkeypatch, Z, sets):
    """RHF of a closed-shell atom in an uncontracted even-tempered basis
    (sets: [(type, exponents)]), XC off, host integrals."""
    import chinium_gb300 as cg
    from chinium_gb300 import scf

    class NoXC:
        EXX = 1.0
        type = 0

        def __init__(self, spin=1):
            pass

        def Read(self, name):
            return self

    monkeypatch.setattr(scf, "ExchangeCorrelation", NoXC)
    types, exps = [], []
    for t, ex in sets:
        types += [t] * len(ex)
        exps += list(ex)
    xyz = np.zeros((1, 3))
    b = cg.Basis.from_shells([Z], xyz, [0] * len(types), types, [1] * len(types), exps, [1.0] * len(exps),
                             normalize=True)
    S, T, V = scf.one_electron(b)

    class NoXCGrid:
        def build(self, xc, D, precision=0):
            return 0.0, [np.zeros((b.nbasis, b.nbasis)) for _ in D]

    ctx = {"basis": b, "S": S, "H": T + V, "jk": scf.JK(scf.repulsion(b, 0.0)), "grid": NoXCGrid(), "Enuc": 0.0,
           "grid_key": ("grid", 1, "HF", "SG-1", 0.0)}
    r = scf.run_scf([Z], xyz, functional="HF", guess="core", context=ctx, conv_energy=1e-11, jk_device="cpu",
                    max_iter=200)
    assert r.converged
    return r.energy


def _even(a0, beta, k):
    return [a0 * beta ** i for i in range(k)]


@pytest.mark.parametrize("Z,sets,limit,window", [
    # numerical Hartree-Fock limits of the atoms; the s (and, for neon, p)
    # even-tempered sets reach them from above within the window
    (2, [(0, _even(0.02, 2.2, 22))], -2.8616799956, 2e-7),
    (4, [(0, _even(0.01, 2.0, 28))], -14.5730231683, 3e-7),
    (10, [(0, _even(0.05, 2.0, 28)), (1, _even(0.04, 2.0, 17))], -128.5470981, 2e-6),
])
def test_closed_shell_atoms_reach_the_hartree_fock_limit(monkeypatch, Z, sets, limit, window):
    """He, Be and Ne RHF in large uncontracted even-tempered s / p bases:
    above the numerical Hartree-Fock limit (variational) and within a few
    1e-7 Eh (He, Be) or 2e-6 Eh (Ne) of it: the host McMurchie-Davidson s and
    p integrals, their J / K contraction and the SCF energy expression against
    an independent physical number."""
    E = _hf_atom(monkeypatch, Z, sets)
    assert limit - 1e-9 < E < limit + window, (Z, E, E - limit)


def test_hartree_fock_energy_is_invariant_under_rigid_motion(monkeypatch):
    """H2O / def2-TZVP (d and f shells on oxygen) rotated at random and
    translated: the overlap matrix changes element by element but the RHF
    energy does not (to 1e-10 Eh), which a wrong solid-harmonic transform
    or d / f integral would break."""
    from scipy.spatial.transform import Rotation
    from chinium_gb300 import molecules as M
    Z, xyz = M.h2o()
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    R = Rotation.random(random_state=3).as_matrix()
    moved = xyz @ R.T + np.array([0.7, -1.3, 2.1])
    r0, S0, _ = _host_hf(monkeypatch, Z, xyz, "def2-tzvp", mult=1)
    r1, S1, _ = _host_hf(monkeypatch, Z, moved, "def2-tzvp", mult=1)
    assert np.abs(S0 - S1).max() > 0.1
    assert np.abs(np.linalg.eigvalsh(S0) - np.linalg.eigvalsh(S1)).max() < 1e-12
    assert abs(r0.energy - r1.energy) < 1e-10, (r0.energy, r1.energy)
