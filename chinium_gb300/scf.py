"""Kohn-Sham SCF driver: the caller of the XC build.

Restates the reference's restricted / unrestricted DIIS SCF
(src/HartreeFockKohnSham/Restricted/SP.cpp:20-81, Unrestricted/SP.cpp:19-104):
per iteration, diagonalise the orthogonalised Fock matrix, form the density,
build Coulomb / exact exchange from the repulsion integrals
(Int4C2E::ContractInts, src/Integral/Int4C2E.cpp:601-683: J from the total
density, K scaled by the functional's EXX fraction), call the XC build, and
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
from ._lib import check, lib
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

    def exchange(self, D):
        return (self.K @ D.ravel()).reshape(self.n, self.n)


class JKDevice:
    """Coulomb and exchange matrices from repulsion integrals resident in HBM
    (two n^2 x n^2 FP64 layouts; each matrix is one matrix-vector product on
    the GPU).  Caller-side plumbing for the SCF: torch only moves and
    multiplies the arrays."""

    def __init__(self, eri):
        import torch
        self.torch = torch
        n = eri.shape[0]
        self.n = n
        t = torch.from_numpy(np.ascontiguousarray(eri)).cuda()
        self.J = t.reshape(n * n, n * n)
        self.K = t.permute(0, 2, 1, 3).contiguous().reshape(n * n, n * n)

    def _mv(self, A, D):
        torch = self.torch
        d = torch.from_numpy(np.ascontiguousarray(D).ravel()).cuda()
        return (A @ d).reshape(self.n, self.n).cpu().numpy()

    def coulomb(self, D):
        return self._mv(self.J, D)

    def exchange(self, D):
        return self._mv(self.K, D)


def make_jk(eri, device):
    if device == "cuda":
        return JKDevice(eri)
    return JK(eri)


class DIIS:
    def __init__(self, size=20):
        self.size = size
        self.F, self.E = [], []

    def push(self, F, err):
        self.F.append(F)
        self.E.append(err)
        if len(self.F) > self.size:
            self.F.pop(0)
            self.E.pop(0)

    def extrapolate(self):
        m = len(self.F)
        if m < 2:
            return self.F[-1]
        B = -np.ones((m + 1, m + 1))
        B[m, m] = 0
        for i in range(m):
            for j in range(m):
                B[i, j] = sum(np.vdot(a, b) for a, b in zip(self.E[i], self.E[j]))
        rhs = np.zeros(m + 1)
        rhs[m] = -1
        try:
            c = np.linalg.solve(B + np.eye(m + 1) * 1e-14 * np.abs(B).max() * (np.arange(m + 1) < m), rhs)[:m]
        except np.linalg.LinAlgError:
            return self.F[-1]
        return [sum(ci * Fi[s] for ci, Fi in zip(c, self.F)) for s in range(len(self.F[0]))]


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
            eri_threshold=1e-12, anchor_every=0, context=None, verbose=False, jk_device="cpu"):
    """Kohn-Sham SCF.  precision: "fp64" (plain XC build every iteration) or
    "mixed" (incremental tensor-core XC builds after an FP64 first build).
    guess: "sap", "core", "learned" (the per-atom-pair network, with the SAP
    guess as fallback: for molecules outside the model's elements / basis, for
    open shells, and when the SCF started from it has not converged within
    half of max_iter), or a density matrix (total for RKS, [Da, Db] for UKS).
    context: reuse integrals and grid from a previous call on the same
    molecule ({"basis","S","H","jk","grid","Enuc"}).
    jk_device: "cpu" (numpy) or "cuda" (repulsion integrals kept in HBM)."""
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
        ctx.update(basis=b, S=S, H=T + Vn, jk=make_jk(repulsion(b, eri_threshold), jk_device),
                   Enuc=M.nuclear_repulsion(Z, xyz))
    key = ("grid", nspin, functional, grid, screen)
    xc = ExchangeCorrelation(spin=nspin).Read(functional)
    if ctx.get("grid_key") != key:
        g = Grid(ctx["basis"], grid, nspin=nspin, screen_threshold=screen)
        g.setType(xc.type)
        g.getAO(0)
        ctx["grid"], ctx["grid_key"] = g, key
    b, S, H, jk, Enuc, g = ctx["basis"], ctx["S"], ctx["H"], ctx["jk"], ctx["Enuc"], ctx["grid"]
    n = b.nbasis
    s_val, s_vec = np.linalg.eigh(S)
    keep = s_val > 1e-8
    X = s_vec[:, keep] / np.sqrt(s_val[keep])
    timings["setup"] = time.perf_counter() - t_start

    def solve(F):
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        return e, X @ Cp

    if isinstance(guess, str) and guess == "learned":
        from . import guess as G
        kw = dict(basis=basis, functional=functional, grid=grid, charge=charge, mult=mult, precision=precision,
                  conv_energy=conv_energy, conv_grad=conv_grad, diis_size=diis_size, screen=screen,
                  eri_threshold=eri_threshold, anchor_every=anchor_every, context=ctx, verbose=verbose,
                  jk_device=jk_device)
        if unrestricted or charge != 0 or not G.supported(Z, b):
            r = run_scf(Z, xyz, guess="sap", max_iter=max_iter, **kw)
            r["guess_used"] = "sap (outside the learned model's scope)"
            return r
        D0 = G.guess_density(G.default_model(), Z, xyz, ctx)
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
            V0 = g.sap_fock()
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
    else:
        Ds = [np.asarray(d, dtype=np.float64) for d in (guess if unrestricted else [guess])]

    diis = DIIS(diis_size)
    E_old = None
    history = []
    converged = False
    exx = xc.EXX
    Vxc_E = 0.0
    for it in range(1, max_iter + 1):
        t0 = time.perf_counter()
        Dtot = Ds[0] if not unrestricted else Ds[0] + Ds[1]
        J = jk.coulomb(Dtot)
        Ks = [jk.exchange(d) for d in Ds] if exx > 0 else [np.zeros((n, n))] * nspin
        timings["jk"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        if precision == "fp64":
            Exc, Vxc = g.build(xc, Ds)
        else:
            anchor = it == 1 or (anchor_every and (it - 1) % anchor_every == 0)
            Dst = np.ascontiguousarray(np.stack([d.T for d in Ds]))
            Vb = np.zeros((nspin, n, n))
            e = ctypes.c_double()
            check(lib().xc_build_incremental(g._h, xc._h, _p(Dst), nspin, int(anchor), ctypes.byref(e), _p(Vb)))
            Exc, Vxc = e.value, [Vb[s].T.copy() for s in range(nspin)]
        timings["xc"] += time.perf_counter() - t0
        if unrestricted:
            Fs = [H + J - exx * Ks[s] + Vxc[s] for s in range(2)]
            E = (np.sum(Dtot * H) + 0.5 * np.sum(Dtot * J) - 0.5 * exx * (np.sum(Ds[0] * Ks[0]) + np.sum(Ds[1] * Ks[1]))
                 + Exc + Enuc)
        else:
            Fs = [H + J - 0.5 * exx * Ks[0] + Vxc[0]]
            E = np.sum(Dtot * H) + 0.5 * np.sum(Dtot * J) - 0.25 * exx * np.sum(Dtot * Ks[0]) + Exc + Enuc
        errs = [X.T @ (F @ D @ S - S @ D @ F) @ X for F, D in zip(Fs, Ds)]
        gmax = max(np.abs(e).max() for e in errs)
        dE = None if E_old is None else E - E_old
        history.append((E, gmax))
        if verbose:
            print("iter %3d  E = %.12f  dE = %s  |grad| = %.3e" % (it, E, "%.3e" % dE if dE is not None else "-", gmax))
        if dE is not None and abs(dE) < conv_energy and gmax < conv_grad:
            converged = True
            break
        E_old = E
        diis.push(Fs, errs)
        Fx = diis.extrapolate()
        t0 = time.perf_counter()
        if unrestricted:
            Ds = []
            for s, occ in enumerate((na, nb)):
                _, C = solve(Fx[s])
                Ds.append(C[:, :occ] @ C[:, :occ].T)
        else:
            _, C = solve(Fx[0])
            Ds = [2 * C[:, :na] @ C[:, :na].T]
        timings["diag"] += time.perf_counter() - t0
    wall = time.perf_counter() - t_start
    return Result(energy=E, converged=converged, iterations=it, wall=wall, timings=timings, D=Ds,
                  history=history, Exc=Exc, context=ctx, nbasis=n,
                  guess_used=guess if isinstance(guess, str) else "caller density")
