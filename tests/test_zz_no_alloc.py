"""The allocation-free entry point (xc_functional_energy_static).

It exists for callers that may not call cudaMalloc / cudaFree: their device
memory belongs to another allocator, or they must not trigger the device-wide
synchronisation those calls imply.  It computes the functional and E_xc on
buffers the caller owns, keeping its only scratch (per-CTA energy partials)
in a fixed array compiled into the library.  This file runs last so that a
failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

import chinium_gb300 as cg
from chinium_gb300 import molecules as M
from chinium_gb300._lib import check, lib

pytestmark = pytest.mark.gpu

E_TOL = 1e-10  # the E_xc bar of the FP64 parity tests


def _density(n, nocc, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(n, nocc)) * 0.1
    A[np.arange(nocc), np.arange(nocc)] += 1.0
    Q, _ = np.linalg.qr(A)
    return 2.0 * Q @ Q.T


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("name,type_,nspin", [("PBE", 1, 1), ("TPSS", 2, 1), ("SVWN5", 0, 2), ("PBE", 1, 2),
                                              ("TPSS", 2, 2)])
def test_static_scratch_entry_matches_grid_path(name, type_, nspin):
    """Restricted and unrestricted (the two-spin offsets n, 2n of rho, sigma,
    tau), LDA / GGA / meta-GGA: the allocation-free entry point against the
    allocating grid path on the same densities, two calls in a row."""
    torch = pytest.importorskip("torch")
    Z, xyz = M.h2o()
    basis = cg.Basis(Z, xyz, "def2-svp")
    grid = cg.Grid(basis, "SG-1", nspin=nspin)
    grid.setType(type_)
    grid.getAO(0)
    xc = cg.ExchangeCorrelation(spin=nspin).Read(name)
    D = _density(basis.nbasis, 5)
    grid.getDensity([D] if nspin == 1 else [0.55 * D, 0.45 * D])
    xc.Evaluate("ev", grid)
    # the existing (allocating) entry points
    E_ref = grid.getEnergy()
    pv = grid.potential_values()
    dv = grid.density_values()
    w = grid.points()["w"]
    n = len(w)
    nsig = 1 if nspin == 1 else 3

    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    d_w, d_rho = dev(w), dev(dv["rho"])
    d_sigma = dev(dv["sigma"]) if type_ >= 1 else None
    d_tau = dev(dv["tau"]) if type_ >= 2 else None
    shapes = {"eps": n, "vrho": nspin * n, "vsigma": nsig * n, "vtau": nspin * n}
    outs = {k: torch.zeros(v, dtype=torch.float64, device="cuda") for k, v in shapes.items()}
    d_E = torch.zeros(1, dtype=torch.float64, device="cuda")
    opt = lambda t: None if t is None else _ptr(t)
    for call in range(2):  # two calls in a row share (and overwrite) the static scratch
        for t in outs.values():
            t.fill_(float("nan"))
        d_E.fill_(float("nan"))
        check(lib().xc_functional_energy_static(xc._h, n, _ptr(d_w), _ptr(d_rho), opt(d_sigma), opt(d_tau),
                                                _ptr(outs["eps"]), _ptr(outs["vrho"]), _ptr(outs["vsigma"]),
                                                _ptr(outs["vtau"]), _ptr(d_E), None))
        torch.cuda.synchronize()
        assert abs(float(d_E.item()) - E_ref) <= E_TOL, (call, float(d_E.item()), E_ref)
        assert np.allclose(outs["eps"].cpu().numpy(), pv["eps"], rtol=1e-13, atol=1e-300)
        assert np.allclose(outs["vrho"].cpu().numpy(), pv["vrho"].ravel(), rtol=1e-13, atol=1e-300)
        if type_ >= 1:
            assert np.allclose(outs["vsigma"].cpu().numpy(), pv["vsigma"].ravel(), rtol=1e-13, atol=1e-300)
        if type_ >= 2:
            assert np.allclose(outs["vtau"].cpu().numpy(), pv["vtau"].ravel(), rtol=1e-13, atol=1e-300)
