"""The CPKS driver's host logic on the CPU: with the XC response switched off
(a stand-in grid and functional whose V_xc and V_xc,U vanish) the
electric-field CPKS of chinium_gb300.cpscf is coupled-perturbed Hartree, whose
polarizability an explicit linear solve of
(e_a - e_i) U_ai + 4 sum_bj (ai|bj) U_bj = -M_ai gives independently (real
integrals, dipoles and Coulomb matrices, all host code)."""
import numpy as np

import chinium_gb300 as cg
from chinium_gb300 import cpscf
from chinium_gb300 import molecules as M
from chinium_gb300.scf import JK, Result, occupations, one_electron, overlap_metric, repulsion


class NoXCGrid:
    """Grid stand-in: V_xc = 0 and V_xc,U = 0 (the calls the driver makes)."""

    def __init__(self, n):
        self.n = n
        self.nmat = 0

    def build(self, xc, D, precision=0):
        return 0.0, [np.zeros((self.n, self.n))]

    def getDensity(self, D):
        pass

    def getDensityU(self, DU):
        self.nmat = len(DU)

    def getFockU(self):
        return [[np.zeros((self.n, self.n)) for _ in range(self.nmat)]]

    def setResponsePrecision(self, p):
        pass


class NoXC:
    EXX = 0.0

    def __init__(self, spin=1):
        pass

    def Read(self, name):
        return self

    def Evaluate(self, order, grid):
        pass


def test_cpks_without_xc_is_coupled_perturbed_hartree(monkeypatch):
    monkeypatch.setattr(cpscf, "ExchangeCorrelation", NoXC)
    Z, xyz = M.h2o()
    b = cg.Basis(Z, xyz, "def2-svp")
    n = b.nbasis
    S, T, V = one_electron(b)
    H = T + V
    eri = repulsion(b)
    ctx = {"basis": b, "S": S, "H": H, "jk": JK(eri), "grid": NoXCGrid(n)}
    na, _ = occupations(Z, 0, 1)
    # a ground state: the core-Hamiltonian orbitals (the CPKS is posed on whatever D it is given)
    X = overlap_metric(S, ctx)[0]
    _, Cp = np.linalg.eigh(X.T @ H @ X)
    C0 = X @ Cp
    D = 2 * C0[:, :na] @ C0[:, :na].T
    scf = Result(D=[D], context=ctx, energy=0.0, converged=True, iterations=0)
    alpha, iters = cpscf.polarizability(Z, xyz, scf, "none", conv=1e-11)
    assert iters < 60
    # the explicit response matrix on the driver's own orbitals: F = H + J(D)
    F = H + ctx["jk"].coulomb(D)
    e, Cq = np.linalg.eigh(X.T @ F @ X)
    C = X @ Cq
    Co, Cv = C[:, :na], C[:, na:]
    nv = n - na
    ovov = np.einsum("pqrs,pa,qi,rb,sj->aibj", eri, Cv, Co, Cv, Co, optimize=True).reshape(nv * na, nv * na)
    A = np.diag((e[na:][:, None] - e[:na][None, :]).ravel()) + 4.0 * ovov
    Md = cpscf.dipole_integrals(b)
    ref = np.zeros((3, 3))
    for l in range(3):
        U = np.linalg.solve(A, -(Cv.T @ Md[l] @ Co).ravel()).reshape(nv, na)
        dD = 2.0 * (Cv @ U @ Co.T + Co @ U.T @ Cv.T)
        for k in range(3):
            ref[k, l] = -np.sum(dD * Md[k])
    assert np.abs(alpha - ref).max() < 1e-8 * np.abs(ref).max(), (alpha, ref)
    assert np.abs(alpha - alpha.T).max() < 1e-8
