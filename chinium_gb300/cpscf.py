"""Coupled-perturbed Kohn-Sham for a static electric field (restricted): the
static dipole polarizability.

This is the electric-field case of the reference's coupled-perturbed solver
(NonIdempotent, src/HartreeFockKohnSham/CoupledPerturbed.cpp:29-160): the
perturbation leaves the basis in place (no overlap derivatives, Ss = 0) and its
skeleton Fock derivative is the dipole operator, so with the occupied-virtual
rotations U of the orbitals C the first-order density and Fock matrices are

    D_U = 2 (C_v U C_o^T + C_o U^T C_v^T)
    F_U = M_k + J(D_U) - exx/2 K(D_U) + V_xc,U(D_U)
    U   = -(C_v^T F_U C_o) / (e_v - e_o)

iterated to self-consistency with DIIS on the rotation residuals (the
reference accelerates with CDIIS).  V_xc,U comes from Grid.getDensityU +
Grid.getFockU (getFockU<u_t>), as in every iteration of CoupledPerturbed.cpp:
131-134, on the ground state of getDensity + Evaluate("ev") + Evaluate("f");
setResponsePrecision(PRECISION_MIXED) puts the per-iteration response on the
tensor cores.  alpha_kl = d mu_k / d F_l = -tr(D_U,l M_k) with the
Hamiltonian H + sum_l F_l M_l (electrons of charge -1 in the field).
"""
import ctypes

import numpy as np

from ._lib import PRECISION_FP64, PRECISION_MIXED, check, lib
from .scf import occupations, overlap_metric, run_scf
from .xc import ExchangeCorrelation


def dipole_integrals(basis, origin=(0.0, 0.0, 0.0)):
    """<mu| r_k - C_k |nu> for k = x, y, z: (3, n, n)."""
    n = basis.nbasis
    M = np.zeros((3, n, n))
    C = np.ascontiguousarray(origin, dtype=np.float64)
    check(lib().xc_dipole(basis._h, C.ctypes.data_as(ctypes.c_void_p), M.ctypes.data_as(ctypes.c_void_p)))
    return M


def ground_state(scf, functional):
    """Orbitals and orbital energies of a converged restricted SCF result
    (its Fock matrix rebuilt once with an FP64 XC build)."""
    ctx = scf.context
    S, H, jk, g = ctx["S"], ctx["H"], ctx["jk"], ctx["grid"]
    xc = ExchangeCorrelation().Read(functional)
    D = scf.D[0]
    _, V = g.build(xc, [D], PRECISION_FP64)
    F = H + jk.coulomb(D) + V[0]
    if xc.EXX > 0:
        F = F - 0.5 * xc.EXX * jk.exchange(D)
    X = overlap_metric(S, ctx)[0]
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    return e, X @ Cp, xc


def polarizability(Z, xyz, scf, functional, precision="fp64", conv=1e-9, max_iter=60, diis_size=8,
                   origin=(0.0, 0.0, 0.0)):
    """Static polarizability tensor (3 x 3, atomic units) by CPKS on a
    converged restricted SCF (a run_scf result for the same functional, with
    conv tight enough for the accuracy wanted).  precision: "fp64" or "mixed" (response densities and
    V_xc,U on the tensor cores, FP64 ground state).  Returns (alpha,
    iterations)."""
    ctx = scf.context
    b, jk, g = ctx["basis"], ctx["jk"], ctx["grid"]
    if scf.D and len(scf.D) != 1:
        raise ValueError("restricted ground states only")
    na, _ = occupations(Z, 0, 1)
    e, C, xc = ground_state(scf, functional)
    Co, Cv = C[:, :na], C[:, na:]
    denom = e[na:][:, None] - e[:na][None, :]
    M = dipole_integrals(b, origin)
    exx = xc.EXX
    # response ground state (Restricted/Hess.cpp:79: Evaluate("f") once before the CPSCF loop)
    g.getDensity([scf.D[0]])
    xc.Evaluate("ev", g)
    xc.Evaluate("f", g)
    g.setResponsePrecision(PRECISION_MIXED if precision == "mixed" else PRECISION_FP64)
    rhs = np.stack([Cv.T @ M[k] @ Co for k in range(3)])
    U = -rhs / denom
    hist_u, hist_r = [], []
    it = 0
    try:
        for it in range(1, max_iter + 1):
            dD = [2.0 * (Cv @ U[k] @ Co.T + Co @ U[k].T @ Cv.T) for k in range(3)]
            g.getDensityU(dD)
            VU = g.getFockU()[0]
            Unew = np.empty_like(U)
            for k in range(3):
                F1 = M[k] + jk.coulomb(dD[k]) + VU[k]
                if exx > 0:
                    F1 = F1 - 0.5 * exx * jk.exchange(dD[k])
                Unew[k] = -(Cv.T @ F1 @ Co) / denom
            r = Unew - U
            err = np.abs(r).max()
            if err < conv:
                U = Unew
                break
            # DIIS on the fixed-point map U -> Unew
            hist_u.append(Unew)
            hist_r.append(r)
            hist_u, hist_r = hist_u[-diis_size:], hist_r[-diis_size:]
            m = len(hist_r)
            B = np.empty((m + 1, m + 1))
            B[-1, :] = B[:, -1] = -1.0
            B[-1, -1] = 0.0
            for i in range(m):
                for j in range(m):
                    B[i, j] = np.sum(hist_r[i] * hist_r[j])
            rhs_d = np.zeros(m + 1)
            rhs_d[-1] = -1.0
            try:
                c = np.linalg.solve(B + np.eye(m + 1) * 1e-14 * np.abs(B).max() * (np.arange(m + 1) < m), rhs_d)[:m]
                U = sum(ci * ui for ci, ui in zip(c, hist_u))
            except np.linalg.LinAlgError:
                U = Unew
    finally:
        g.setResponsePrecision(PRECISION_FP64)
    dD = [2.0 * (Cv @ U[k] @ Co.T + Co @ U[k].T @ Cv.T) for k in range(3)]
    alpha = np.array([[-np.sum(dD[l] * M[k]) for l in range(3)] for k in range(3)])
    return alpha, it


def finite_field_polarizability(Z, xyz, scf, functional, axis, field=4e-3, conv_energy=1e-12, conv_grad=1e-8,
                                **kw):
    """alpha along one axis as -d^2 E / d F^2 of SCF energies with H + F M_axis:
    central differences at F and F/2 combined by Richardson extrapolation
    (test reference for polarizability).  kw: the grid / screen / jk_device of
    the SCF that made scf, so that its context (integrals, grid) is reused."""
    ctx = scf.context
    M = dipole_integrals(ctx["basis"])

    def energy(F):
        c2 = dict(ctx)
        c2["H"] = ctx["H"] + F * M[axis]
        r = run_scf(Z, xyz, guess=scf.D[0], context=c2, conv_energy=conv_energy, conv_grad=conv_grad,
                    functional=functional, **kw)
        if not r.converged:
            raise RuntimeError("finite-field SCF did not converge")
        return r.energy

    E0 = energy(0.0)
    d = []
    for h in (field, 0.5 * field):
        d.append(-(energy(h) + energy(-h) - 2.0 * E0) / (h * h))
    return (4.0 * d[1] - d[0]) / 3.0
