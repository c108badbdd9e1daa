"""Kohn-Sham SCF driver: the caller of the XC build.

Restates the reference's restricted / unrestricted DIIS SCF
(src/HartreeFockKohnSham/Restricted/SP.cpp:20-81, Unrestricted/SP.cpp:19-104):
per iteration, diagonalise the orthogonalised Fock matrix, form the density,
build Coulomb / exact exchange from the repulsion integrals (the library's
GPU engine, the role of Int4C2E::CalculateIntegrals + ContractInts,
src/Integral/Int4C2E.cpp:567-683: J from the total density, K scaled by the
functional's EXX fraction), call the XC build, and
extrapolate with Pulay's commutator DIIS (src/DIIS/CDIIS.cpp:24-47).  The
energy expression is the reference's E = D.(Hcore + F_hf) + E_xc
(Restricted/SP.cpp:59) written with the total density.

Initial guesses: the superposition of atomic potentials
(GuessSCF.cpp:17-99, through the XC library's SAP V assembly), the core
Hamiltonian, or a caller-supplied density matrix (the learned guess).

Convergence: |dE| < conv_energy (1e-8 Eh by default) and
max |X^T (F D S - S D F) X| < conv_grad (the reference's 1e-6 bar).
"""
import ctypes
import time

import numpy as np
import scipy.linalg

from . import molecules as M
from ._lib import PRECISION_FP64, PRECISION_MIXED, check, lib
from .xc import Basis, ExchangeCorrelation, Grid


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def one_electron(basis):
    n = basis.nbasis
    S, T, V = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
    check(lib().xc_int1e(basis._h, _p(S), _p(T), _p(V)))
    return S, T, V


def repulsion(basis, threshold=1e-12):
    n = basis.nbasis
    eri = np.zeros(n ** 4)
    check(lib().xc_eri(basis._h, _p(eri), ctypes.c_double(threshold)))
    return eri.reshape(n, n, n, n)


class JK:
    """Coulomb and exchange matrices from in-core repulsion integrals."""

    def __init__(self, eri):
        n = eri.shape[0]
        self.n = n
        self.J = eri.reshape(n * n, n * n)
        self.K = np.ascontiguousarray(eri.transpose(0, 2, 1, 3)).reshape(n * n, n * n)

    def coulomb(self, D):
        return (self.J @ D.ravel()).reshape(self.n, self.n)

    # the host contraction has nothing to overlap: begin computes, end returns
    def coulomb_begin(self, D):
        return self.coulomb(D)

    def coulomb_end(self, h):
        return h

    def exchange(self, D):
        return (self.K @ D.ravel()).reshape(self.n, self.n)


class JKEngine:
    """Coulomb and exchange matrices from the library's GPU integral engine
    (include/chinium_int.h, xc_jk_*: the reference's Int4C2E): the screened
    unique integrals are computed on the GPU once and kept in HBM, or
    recomputed per build when they do not fit, and every build contracts them
    with the density matrices.  begin() enqueues J (of the summed densities)
    and, when asked, K of each density on the engine's own stream and returns
    at once, so that the XC build can run meanwhile; end() waits."""

    def __init__(self, basis, threshold=1e-14, max_bytes=0.0):
        import torch
        self.torch = torch
        self.n = basis.nbasis
        h = ctypes.c_void_p()
        check(lib().xc_jk_create(basis._h, float(threshold), float(max_bytes), ctypes.byref(h)))
        self._h = h
        self.stream = torch.cuda.Stream()
        check(lib().xc_jk_set_stream(h, ctypes.c_void_p(self.stream.cuda_stream)))
        self._pinned = None  # page-locked upload buffer, reused (pinning per call costs ~1 ms)

    def info(self):
        nq, ni, ic = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
        check(lib().xc_jk_info(self._h, ctypes.byref(nq), ctypes.byref(ni), ctypes.byref(ic)))
        return {"quartets": nq.value, "integrals": ni.value, "incore": bool(ic.value)}

    def begin(self, Ds, want_k):
        torch = self.torch
        n, m = self.n, len(Ds)
        if self._pinned is None or self._pinned.shape[0] < m:
            self.stream.synchronize()
            self._pinned = torch.empty((m, n, n), dtype=torch.float64).pin_memory()
        self.stream.synchronize()  # the previous upload from the buffer has completed
        host = self._pinned[:m]
        for i, Dm in enumerate(Ds):
            host[i].numpy()[...] = Dm
        with torch.cuda.stream(self.stream):
            d = host.cuda(non_blocking=True)
            J = torch.empty((m, n, n), dtype=torch.float64, device="cuda")
            K = torch.empty((m, n, n), dtype=torch.float64, device="cuda") if want_k else None
        ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
        check(lib().xc_jk_build_device(self._h, m, ptr(d), ptr(J), ptr(K)))
        return d, J, K

    def end(self, h):
        d, J, K = h
        self.stream.synchronize()
        Jh = J.cpu().numpy().sum(axis=0)
        Ks = [K[s].cpu().numpy() for s in range(K.shape[0])] if K is not None else None
        return Jh, Ks

    def coulomb(self, D):
        return self.end(self.begin([D], False))[0]

    def exchange(self, D):
        return self.end(self.begin([D], True))[1][0]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xc_jk_destroy(h)
            self._h = None


def overlap_metric(S, ctx=None):
    """(X, S^-1/2, S^1/2) of the overlap matrix: X the canonical
    orthogonaliser (eigenvectors with eigenvalue > 1e-8, scaled), the other
    two over the full spectrum.  Kept in ctx (one molecule) when given."""
    if ctx is not None and "S_metric" in ctx:
        return ctx["S_metric"]
    w, V = np.linalg.eigh(S)
    keep = w > 1e-8
    m = (V[:, keep] / np.sqrt(w[keep]), (V * w ** -0.5) @ V.T, (V * w ** 0.5) @ V.T)
    if ctx is not None:
        ctx["S_metric"] = m
        ctx["S_min"] = float(w[0])  # smallest overlap eigenvalue (near-linear dependence)
    return m


def make_jk(basis, device, eri_threshold=1e-12):
    """J/K provider of an SCF: "engine" (or "cuda"): the library's GPU
    integrals and contraction; "cpu": the full host integral tensor with numpy
    contractions (small molecules, host-side checks)."""
    if device in ("engine", "cuda"):
        return JKEngine(basis)
    if device == "cpu":
        return JK(repulsion(basis, eri_threshold))
    raise ValueError("jk_device must be 'engine', 'cuda' or 'cpu'")


class DIIS:
    """Pulay's commutator DIIS (src/DIIS/CDIIS.cpp:24-47); the error inner
    products are kept from one push to the next (each push adds one row).
    The history also keeps each iterate's densities and energy, which the
    ADIIS stage that precedes it uses (the reference's ADIIS run hands its
    history to CDIIS, Restricted/SP.cpp:75-79)."""

    def __init__(self, size=20):
        self.size = size
        self.F, self.E, self.D, self.En = [], [], [], []
        self.G = np.zeros((0, 0))

    def push(self, F, err, D=None, energy=None):
        self.F.append(F)
        self.E.append(err)
        self.D.append(D)
        self.En.append(energy)
        row = np.array([sum(np.vdot(a, b) for a, b in zip(e, err)) for e in self.E])
        m = len(self.E)
        G = np.zeros((m, m))
        G[:m - 1, :m - 1] = self.G
        G[m - 1, :] = row
        G[:, m - 1] = row
        self.G = G
        if len(self.F) > self.size:
            for lst in (self.F, self.E, self.D, self.En):
                lst.pop(0)
            self.G = self.G[1:, 1:]

    def extrapolate(self):
        m = len(self.F)
        if m < 2:
            return self.F[-1]
        B = -np.ones((m + 1, m + 1))
        B[m, m] = 0
        B[:m, :m] = self.G
        rhs = np.zeros(m + 1)
        rhs[m] = -1
        try:
            c = np.linalg.solve(B + np.eye(m + 1) * 1e-14 * np.abs(B).max() * (np.arange(m + 1) < m), rhs)[:m]
        except np.linalg.LinAlgError:
            return self.F[-1]
        return [sum(ci * Fi[s] for ci, Fi in zip(c, self.F)) for s in range(len(self.F[0]))]

    def extrapolate_adiis(self):
        """Augmented DIIS (Hu and Yang, J. Chem. Phys. 132, 054109 (2010);
        src/DIIS/AEDIIS.cpp:29-104): weights x on the simplex minimising
        x.(A + B x / 2) with A_i = (D_i - D_n).F_n and B_ij = (D_i - D_n).(F_j
        - F_n), summed over the spin matrices (n the latest iterate), from
        the reference's start (0.9 on the latest, the rest shared)."""
        m = len(self.F)
        if m < 2 or any(d is None for d in self.D):
            return self.F[-1]
        ns = len(self.F[0])
        A = np.zeros(m)
        B = np.zeros((m, m))
        for s in range(ns):
            Dn, Fn = self.D[-1][s], self.F[-1][s]
            dD = [self.D[i][s] - Dn for i in range(m)]
            dF = [self.F[j][s] - Fn for j in range(m)]
            A += np.array([np.vdot(dD[i], Fn) for i in range(m)])
            B += np.array([[np.vdot(dD[i], dF[j]) for j in range(m)] for i in range(m)])
        x = minimise_on_simplex(A, B)
        return [sum(xi * Fi[s] for xi, Fi in zip(x, self.F)) for s in range(ns)]


def project_simplex(v):
    """Euclidean projection onto {x >= 0, sum x = 1} (sort-based)."""
    u = np.sort(v)[::-1]
    css = np.cumsum(u) - 1.0
    k = np.nonzero(u * np.arange(1, len(v) + 1) > css)[0][-1]
    return np.maximum(v - css[k] / (k + 1), 0.0)


def minimise_on_simplex(A, B, iters=400):
    """min_x x.A + x.B x / 2 over the simplex: accelerated projected gradient
    (FISTA) from the reference's start, keeping the best iterate (B need not
    be positive definite).  Small dense numpy only (m <= DIIS size)."""
    m = len(A)
    Bs = 0.5 * (B + B.T)
    L = max(np.abs(np.linalg.eigvalsh(Bs)).max(), 1e-12)
    f = lambda x: x @ A + 0.5 * x @ Bs @ x
    x = np.full(m, 0.1 / (m - 1))
    x[-1] = 0.9
    y, t, best, fbest = x.copy(), 1.0, x.copy(), f(x)
    for _ in range(iters):
        xn = project_simplex(y - (A + Bs @ y) / L)
        tn = 0.5 * (1.0 + np.sqrt(1.0 + 4.0 * t * t))
        y = xn + ((t - 1.0) / tn) * (xn - x)
        step = np.abs(xn - x).max()
        x, t = xn, tn
        fx = f(x)
        if fx < fbest:
            best, fbest = x.copy(), fx
        if step < 1e-12:
            break
    return best


def cayley_update(C, F, nocc):
    """One orbital update without diagonalisation: the occupied-virtual block
    of F in the current orbitals C (S-orthonormal columns) gives first-order
    rotation angles kappa_ai = -F_ai / (F_aa - F_ii), applied as the exactly
    orthogonal Cayley transform U = (1 - K/2)^-1 (1 + K/2) of the
    antisymmetric K = [[0, -kappa^T], [kappa, 0]].  At the SCF fixed point
    (F_ai = 0) it leaves C unchanged, so the converged state is the one a full
    diagonalisation reaches; the SCF uses it once the DIIS error is small.
    With a = kappa / 2 and W = (1 + a^T a)^-1 (occupied x occupied), the
    block inverse of 1 - K/2 gives U in closed form,
        U_oo = 2 W - 1,  U_vo = 2 a W,  U_ov = -2 W a^T,  U_vv = 1 - 2 a W a^T,
    so the update costs one F C product and occupied-sized solves:
    C_o' = 2 G W - C_o and C_v' = C_v - (C_o' + C_o) a^T with G = C_o + C_v a.
    Returns None when a virtual orbital's diagonal energy is not above every
    occupied one (within 1e-3 Eh): the occupations would no longer follow the
    aufbau order, and the caller diagonalises instead."""
    m = C.shape[1]
    if nocc == 0 or nocc == m:
        return C.copy()  # an empty or full spin channel: no occupied-virtual block to rotate
    Co, Cv = C[:, :nocc], C[:, nocc:]
    FC = F @ C
    e_o = np.einsum("ij,ij->j", Co, FC[:, :nocc])
    e_v = np.einsum("ij,ij->j", Cv, FC[:, nocc:])
    if nocc < m and e_v.min() <= e_o.max() + 1e-3:
        return None  # the occupied set is no longer the lowest: the caller diagonalises (aufbau)
    a = -0.5 * (Cv.T @ FC[:, :nocc]) / (e_v[:, None] - e_o[None, :])
    W = np.linalg.inv(np.eye(nocc) + a.T @ a)
    Co_new = 2.0 * (Co + Cv @ a) @ W - Co
    Cv_new = Cv - (Co_new + Co) @ a.T
    return np.hstack([Co_new, Cv_new])


class Result(dict):
    __getattr__ = dict.__getitem__


def occupations(Z, charge, mult):
    ne = int(sum(Z)) - charge
    nu = mult - 1
    if (ne - nu) % 2:
        raise ValueError("charge and multiplicity are inconsistent")
    nb = (ne - nu) // 2
    return nb + nu, nb


def run_scf(Z, xyz, basis="def2-svp", functional="PBE", grid="SG-1", charge=0, mult=1, precision="fp64",
            guess="sap", conv_energy=1e-8, conv_grad=1e-6, max_iter=100, diis_size=20, screen=0.0,
            eri_threshold=1e-12, anchor_every=0, context=None, verbose=False, jk_device="engine", anchor="fp64",
            adiis_until=1e-1, rotate_below=1e-1, callback=None, reanchor_above=1.0, fp32_potentials=True,
            orbitals=None):
    """Kohn-Sham SCF.  precision: "fp64" (plain XC build every iteration) or
    "mixed" (incremental tensor-core XC builds after a first build that sets
    the references: anchor "fp64", a full FP64 build, "density", FP64
    densities, functional and E_xc with V_xc on the tensor cores (V's error
    moves the converged energy only at second order), or "mixed", a full
    tensor-core build, whose density error stays in E_xc at first order).
    fp32_potentials: the incremental builds' functional takes FP32 potentials
    where the density is above the mixed config's func_float_above (FP64
    energy density everywhere), as a full mixed build does; False keeps the
    potentials in FP64 too.
    guess: "sap", "core", "learned" (the per-atom-pair network, with the SAP
    guess as fallback: for molecules outside the model's elements / basis, for
    open shells, and when the SCF started from it has not converged within
    half of max_iter), or a density matrix (total for RKS, [Da, Db] for UKS).
    orbitals: with a density guess, S-orthonormal orbitals whose occupied
    columns (first) span it ([C] for RKS, [Ca, Cb] for UKS), so that the first
    update may be a rotation (the learned guess's natural orbitals).
    context: reuse integrals and grid from a previous call on the same
    molecule ({"basis","S","H","jk","grid","Enuc"}).
    jk_device: "engine" (alias "cuda": integrals computed on the GPU, kept in
    HBM and contracted there by the library, JKEngine) or "cpu" (the full
    host integral tensor, numpy contraction; small molecules).
    adiis_until: ADIIS extrapolation while the largest commutator element is
    above this (the reference's 1e-1), CDIIS below; 0 = CDIIS throughout.
    rotate_below: once that element is below this, new orbitals come from a
    Cayley rotation of the previous ones (cayley_update) instead of a full
    diagonalisation; 0 = always diagonalise.
    callback: called every iteration as callback(it, Ds, Exc, Vxc, E) (monitoring).
    reanchor_above: mixed precision re-anchors the incremental XC build when a
    density element changed by more than this since the previous build."""
    t_start = time.perf_counter()
    timings = {"setup": 0.0, "xc": 0.0, "jk": 0.0, "diag": 0.0}
    na, nb = occupations(Z, charge, mult)
    unrestricted = mult != 1
    nspin = 2 if unrestricted else 1
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    ctx = context if context is not None else {}
    if "basis" not in ctx:
        b = Basis(Z, xyz, basis)
        S, T, Vn = one_electron(b)
        ctx.update(basis=b, S=S, H=T + Vn, jk=make_jk(b, jk_device, eri_threshold), Enuc=M.nuclear_repulsion(Z, xyz))
    key = ("grid", nspin, functional, grid, screen)
    xc = ExchangeCorrelation(spin=nspin).Read(functional)
    if ctx.get("grid_key") != key:
        g = Grid(ctx["basis"], grid, nspin=nspin, screen_threshold=screen)
        g.setType(xc.type)
        g.getAO(0)
        if jk_device in ("cuda", "engine"):
            # the XC build on its own stream, so that the device J of the same
            # iteration (torch's or the engine's stream) runs alongside it
            import torch
            torch.cuda.synchronize()
            # a higher priority than the J/K stream: the XC build is the longer of the two
            ctx["grid_stream"] = torch.cuda.Stream(priority=-1)
            g.set_stream(ctx["grid_stream"].cuda_stream)
        ctx["grid"], ctx["grid_key"] = g, key
    b, S, H, jk, Enuc, g = ctx["basis"], ctx["S"], ctx["H"], ctx["jk"], ctx["Enuc"], ctx["grid"]
    n = b.nbasis
    X = overlap_metric(S, ctx)[0]
    SX = S @ X
    timings["setup"] = time.perf_counter() - t_start

    def solve(F):
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        return e, X @ Cp

    if isinstance(guess, str) and guess == "learned":
        from . import guess as G
        kw = dict(basis=basis, functional=functional, grid=grid, charge=charge, mult=mult, precision=precision,
                  conv_energy=conv_energy, conv_grad=conv_grad, diis_size=diis_size, screen=screen,
                  eri_threshold=eri_threshold, anchor_every=anchor_every, context=ctx, verbose=verbose,
                  jk_device=jk_device, anchor=anchor, adiis_until=adiis_until, rotate_below=rotate_below,
                  callback=callback, reanchor_above=reanchor_above, fp32_potentials=fp32_potentials)
        if unrestricted or charge != 0 or not G.supported(Z, b):
            r = run_scf(Z, xyz, guess="sap", max_iter=max_iter, **kw)
            r["guess_used"] = "sap (outside the learned model's scope)"
            return r
        # the density alone: rotating from its natural orbitals in the first
        # iteration saves one diagonalisation but costs iterations ((H2O)_8: +1.25)
        D0 = G.guess_density(G.default_model(), Z, xyz, ctx, precision=precision)
        r = run_scf(Z, xyz, guess=D0, max_iter=max(1, max_iter // 2), **kw)
        if r.converged:
            r["guess_used"] = "learned"
            r["wall"] += timings["setup"]
            return r
        r2 = run_scf(Z, xyz, guess="sap", max_iter=max_iter, **kw)
        r2["guess_used"] = "sap (learned start did not converge in %d iterations)" % r.iterations
        return r2

    # initial guess
    if isinstance(guess, str):
        if guess == "sap":
            # the tensor-core SAP matrix (FP32-level error) only when the overlap is well
            # conditioned: the orthogonaliser amplifies an error in V by 1 / s_min
            tc_sap = precision == "mixed" and ctx.get("S_min", 0.0) >= 1e-3
            V0 = g.sap_fock(PRECISION_MIXED if tc_sap else PRECISION_FP64)
            F0 = H + V0
        elif guess == "core":
            F0 = H
        else:
            raise ValueError("unknown guess")
        _, C = solve(F0)
        if unrestricted:
            Ds = [C[:, :na] @ C[:, :na].T, C[:, :nb] @ C[:, :nb].T]
        else:
            Ds = [2 * C[:, :na] @ C[:, :na].T]
        C_init = [C] * nspin
    else:
        Ds = [np.asarray(d, dtype=np.float64) for d in (guess if unrestricted else [guess])]
        C_init = None if orbitals is None else [np.asarray(c, dtype=np.float64) for c in orbitals]
        if C_init is not None and len(C_init) != nspin:
            raise ValueError("orbitals: one matrix per spin")

    anchors = {"fp64": 1, "density": 2, "mixed": 3}
    if anchor not in anchors:
        raise ValueError("anchor must be 'fp64', 'density' or 'mixed'")
    anchor_code = anchors[anchor]
    incr_code = 16 if fp32_potentials else 0  # XC_INCREMENTAL_FP32_POTENTIALS
    diis = DIIS(diis_size)
    Cs = C_init  # orbitals of the last update (per spin)
    D_ref = None  # densities of the last XC build (the incremental reference)
    E_old = None
    history = []
    converged = False
    exx = xc.EXX
    Vxc_E = 0.0
    for it in range(1, max_iter + 1):
        t0 = time.perf_counter()
        Dtot = Ds[0] if not unrestricted else Ds[0] + Ds[1]
        if isinstance(jk, JKEngine):  # J and K on the GPU engine's stream, overlapping the XC build below
            J_pending = jk.begin(Ds, exx > 0)
        else:
            J_pending = jk.coulomb_begin(Dtot)  # overlaps the XC build below
            Ks = [jk.exchange(d) for d in Ds] if exx > 0 else [np.zeros((n, n))] * nspin
        timings["jk"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        if precision == "fp64":
            Exc, Vxc = g.build(xc, Ds)
        else:
            # re-anchor after a large density change: an incremental build's error scales with
            # the change (max |D - D_ref|), and stays in the reconstructed densities
            reset = (it == 1 or (anchor_every and (it - 1) % anchor_every == 0)
                     or max(np.abs(d - r).max() for d, r in zip(Ds, D_ref)) > reanchor_above)
            D_ref = [d.copy() for d in Ds]
            if reset:
                timings["anchors"] = timings.get("anchors", 0) + 1
            Dst = np.ascontiguousarray(np.stack([d.T for d in Ds]))
            Vb = np.zeros((nspin, n, n))
            e = ctypes.c_double()
            code = (anchor_code if reset else 0) | incr_code
            check(lib().xc_build_incremental(g._h, xc._h, _p(Dst), nspin, code, ctypes.byref(e), _p(Vb)))
            Exc, Vxc = e.value, [Vb[s].T.copy() for s in range(nspin)]
        timings["xc"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        if isinstance(jk, JKEngine):
            J, Ks = jk.end(J_pending)
            if Ks is None:
                Ks = [np.zeros((n, n))] * nspin
        else:
            J = jk.coulomb_end(J_pending)
        timings["jk"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        HJ = H + J
        if unrestricted:
            Fs = [HJ + Vxc[s] - exx * Ks[s] if exx else HJ + Vxc[s] for s in range(2)]
            E = (np.vdot(Dtot, H) + 0.5 * np.vdot(Dtot, J) - 0.5 * exx * (np.vdot(Ds[0], Ks[0]) + np.vdot(Ds[1], Ks[1]))
                 + Exc + Enuc)
        else:
            Fs = [HJ + Vxc[0] - 0.5 * exx * Ks[0] if exx else HJ + Vxc[0]]
            E = np.vdot(Dtot, H) + 0.5 * np.vdot(Dtot, J) - 0.25 * exx * np.vdot(Dtot, Ks[0]) + Exc + Enuc
        errs = []
        for F, D in zip(Fs, Ds):
            # X^T (F D S - S D F) X; S D F = (F D S)^T for symmetric F, D, S
            Mc = X.T @ (F @ (D @ SX))
            errs.append(Mc - Mc.T)
        gmax = max(np.abs(e).max() for e in errs)
        dE = None if E_old is None else E - E_old
        timings["fock"] = timings.get("fock", 0.0) + time.perf_counter() - t0
        history.append((E, gmax))
        if callback is not None:
            callback(it, Ds, Exc, Vxc, E)
        if verbose:
            print("iter %3d  E = %.12f  dE = %s  |grad| = %.3e" % (it, E, "%.3e" % dE if dE is not None else "-", gmax))
        if dE is not None and abs(dE) < conv_energy and gmax < conv_grad:
            converged = True
            break
        E_old = E
        t0 = time.perf_counter()
        diis.push(Fs, errs, Ds, E)
        Fx = diis.extrapolate_adiis() if adiis_until > 0 and gmax > adiis_until else diis.extrapolate()
        timings["diis"] = timings.get("diis", 0.0) + time.perf_counter() - t0
        t0 = time.perf_counter()
        occs = (na, nb) if unrestricted else (na,)
        rotate = rotate_below > 0 and gmax < rotate_below and Cs is not None
        new = [cayley_update(Cs[s], Fx[s], occ) if rotate else None for s, occ in enumerate(occs)]
        Cs = [c if c is not None else solve(Fx[s])[1] for s, c in enumerate(new)]
        timings["rotations"] = timings.get("rotations", 0) + sum(c is not None for c in new)
        Ds = [C[:, :occ] @ C[:, :occ].T for C, occ in zip(Cs, occs)]
        if not unrestricted:
            Ds = [2 * Ds[0]]
        timings["diag"] += time.perf_counter() - t0
    wall = time.perf_counter() - t_start
    return Result(energy=E, converged=converged, iterations=it, wall=wall, timings=timings, D=Ds,
                  history=history, Exc=Exc, context=ctx, nbasis=n,
                  guess_used=guess if isinstance(guess, str) else "caller density")
