"""SCF through the XC build (GPU): the caller of the path, as the reference's
DIIS drivers call it once per iteration."""
import numpy as np
import pytest

from chinium_gb300 import molecules as M
from chinium_gb300.scf import run_scf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("functional", ["PBE", "B3LYP", "TPSS"])
def test_rks_h2o_converges_and_mixed_matches_fp64(functional):
    Z, xyz = M.h2o()
    r64 = run_scf(Z, xyz, functional=functional, precision="fp64")
    assert r64.converged and r64.iterations < 40
    rmx = run_scf(Z, xyz, functional=functional, precision="mixed", context=r64.context)
    assert rmx.converged
    print("%s: E64 %.10f  Emixed %.10f  dE %.2e  iters %d/%d" % (functional, r64.energy, rmx.energy,
                                                              rmx.energy - r64.energy, r64.iterations, rmx.iterations))
    # incremental tensor-core builds: converged energy within 1e-6 Eh of the FP64 path
    assert abs(rmx.energy - r64.energy) < 1e-6
    # references from FP64 densities with a tensor-core V
    rd = run_scf(Z, xyz, functional=functional, precision="mixed", anchor="density", context=r64.context)
    assert rd.converged and abs(rd.energy - r64.energy) < 1e-6
    # physically sensible total energy for water in this basis
    assert -77.0 < r64.energy < -75.5


def test_uks_h2o_cation():
    Z, xyz = M.h2o()
    r = run_scf(Z, xyz, functional="PBE", charge=1, mult=2, precision="fp64", max_iter=150)
    assert r.converged
    rm = run_scf(Z, xyz, functional="PBE", charge=1, mult=2, precision="mixed", context=r.context, max_iter=150)
    assert rm.converged and abs(rm.energy - r.energy) < 1e-6
    Da, Db = r.D
    S = r.context["S"]
    assert np.trace(Da @ S) == pytest.approx(5.0, abs=1e-8)
    assert np.trace(Db @ S) == pytest.approx(4.0, abs=1e-8)


def test_sap_guess_beats_core_guess():
    Z, xyz = M.h2o()
    r_sap = run_scf(Z, xyz, functional="PBE", guess="sap")
    r_core = run_scf(Z, xyz, functional="PBE", guess="core", context=r_sap.context)
    assert r_sap.converged and r_core.converged
    assert abs(r_sap.energy - r_core.energy) < 1e-7
    assert r_sap.iterations <= r_core.iterations


def test_gpu_jk_engine_matches_host_jk_in_scf():
    """J/K from the GPU integral engine give the same SCF as the host
    integral tensor (B3LYP: Coulomb and exact exchange)."""
    pytest.importorskip("torch")
    Z, xyz = M.h2o()
    r_cpu = run_scf(Z, xyz, functional="B3LYP", jk_device="cpu", eri_threshold=0.0)
    r_gpu = run_scf(Z, xyz, functional="B3LYP", jk_device="engine")
    assert r_cpu.converged and r_gpu.converged
    assert abs(r_cpu.energy - r_gpu.energy) < 1e-9


def test_engine_coulomb_and_exchange_match_host():
    pytest.importorskip("torch")
    from chinium_gb300.scf import JK, JKEngine, repulsion
    from chinium_gb300.xc import Basis
    Z, xyz = M.h2o()
    b = Basis(Z, xyz, "def2-svp")
    rng = np.random.default_rng(5)
    D = rng.normal(size=(24, 24))
    D = D + D.T
    host, dev = JK(repulsion(b, 0.0)), JKEngine(b)
    assert np.abs(dev.coulomb(D) - host.coulomb(D)).max() < 1e-11
    assert np.abs(dev.exchange(D) - host.exchange(D)).max() < 1e-11


def test_mixed_scf_with_learned_guess_uses_tensor_core_sap():
    """precision="mixed" builds the learned guess's SAP base on the tensor
    cores; the SCF still converges to the FP64 energy."""
    Z, xyz = M.water_clusters(1, seed=99, kmin=2, kmax=2)[0]
    r64 = run_scf(Z, xyz, functional="PBE", precision="fp64", jk_device="engine")
    rl = run_scf(Z, xyz, functional="PBE", precision="mixed", guess="learned", anchor="density",
                 context=r64.context, jk_device="engine")
    assert rl.converged and rl.guess_used == "learned"
    assert abs(rl.energy - r64.energy) < 1e-6


def test_incremental_builds_are_stationary_with_empty_tiles():
    """A water trimer on SG-1 whose grid has a tile that keeps no basis chunk.
    Forty incremental builds at an unchanged density must return the
    anchor's energy every time: no density kernel writes that tile's points,
    and nothing may accumulate there from one call to the next (it once
    doubled per call, which stalled longer SCFs)."""
    import ctypes
    import chinium_gb300 as cg
    from chinium_gb300._lib import check, lib
    Z2, xyz2 = M.water_clusters(24, seed=1, kmin=2, kmax=8)[5]
    r = run_scf(Z2, xyz2, functional="PBE", precision="fp64", max_iter=3)
    g = r.context["grid"]
    xc = cg.ExchangeCorrelation().Read("PBE")
    n = r.nbasis
    D = np.ascontiguousarray(r.D[0].T)[None]
    V = np.zeros((1, n, n))
    e = ctypes.c_double()
    Es = []
    for it in range(40):
        check(lib().xc_build_incremental(g._h, xc._h, ctypes.c_void_p(D.ctypes.data), 1, 2 if it == 0 else 0,
                                         ctypes.byref(e), ctypes.c_void_p(V.ctypes.data)))
        Es.append(e.value)
    assert g.info()["mixed_empty_tiles"] > 0
    assert max(abs(x - Es[0]) for x in Es) < 1e-10


def test_incremental_anchor_kinds_and_fp32_potentials():
    """xc_build_incremental's anchors on (H2O)_3 PBE/SG-1: anchor 3 returns
    the full tensor-core build's E_xc and V_xc; after each anchor, an
    incremental build at a perturbed density is checked against the FP64
    build there: anchor 2 (FP64 densities) to 1e-8 Eh in E_xc (the tensor
    cores only see the change, elements of 2e-3 here), anchor 3 to the
    tensor-core density's own 1e-6, and XC_INCREMENTAL_FP32_POTENTIALS
    moves E_xc by less than 1e-9 Eh (its E stays FP64 arithmetic) while V_xc
    takes FP32-level noise only."""
    import ctypes
    import chinium_gb300 as cg
    from chinium_gb300._lib import check, lib, PRECISION_MIXED
    Z, xyz = M.water_clusters(1, seed=3, kmin=3, kmax=3)[0]
    r = run_scf(Z, xyz, functional="PBE", precision="fp64", max_iter=4)
    g = r.context["grid"]
    xc = cg.ExchangeCorrelation().Read("PBE")
    n = r.nbasis
    D0 = r.D[0]
    P = np.random.default_rng(0).normal(size=(n, n)) * 1e-3
    D1 = D0 + P + P.T

    def inc(D, code):
        Dc = np.ascontiguousarray(D.T)[None]
        V = np.zeros((1, n, n))
        e = ctypes.c_double()
        check(lib().xc_build_incremental(g._h, xc._h, ctypes.c_void_p(Dc.ctypes.data), 1, code, ctypes.byref(e),
                                         ctypes.c_void_p(V.ctypes.data)))
        return e.value, V[0].T

    Em, Vm = g.build(xc, [D0], precision=PRECISION_MIXED)
    E3, V3 = inc(D0, 3)
    assert E3 == Em and np.abs(V3 - Vm[0]).max() < 1e-12
    E64, V64 = g.build(xc, [D1])
    V64 = V64[0]
    # anchor 2's float-float densities with the FP64 functional: E_xc as the FP64 build
    E2, _ = inc(D1, 2)
    assert abs(E2 - E64) < 1e-10, E2 - E64
    out = {}
    for anchor in (2, 3):
        for flag in (0, 16):
            inc(D0, anchor)
            out[anchor, flag] = inc(D1, flag)
    for (anchor, flag), (E, V) in out.items():
        print("anchor %d flag %2d: dE %.2e max|dV| %.2e" % (anchor, flag, E - E64, np.abs(V - V64).max()))
    assert abs(out[2, 0][0] - E64) < 1e-8 and abs(out[2, 16][0] - E64) < 1e-8
    assert abs(out[3, 0][0] - E64) < 1e-6 and abs(out[3, 16][0] - E64) < 1e-6
    assert abs(out[2, 16][0] - out[2, 0][0]) < 1e-9
    assert np.abs(out[2, 16][1] - V64).max() < 1e-5
    with pytest.raises(Exception):
        inc(D1, 4)


@pytest.mark.parametrize("functional,charge,mult", [("SVWN5", 0, 1), ("PBE", 0, 1), ("B3LYP", 0, 1), ("TPSS", 0, 1),
                                                    ("R2SCAN", 0, 1), ("PBE", 1, 2), ("B3LYP", 1, 2), ("TPSS", 1, 2)])
def test_float_float_energy_density_matches_fp64(functional, charge, mult):
    """The mixed functional's energy density in float-float arithmetic (the
    FP32-pair scalar of the functional library: its exp, log, cbrt, sqrt,
    division) against FP64 on the same reconstructed densities: two
    incremental builds after one anchor, one with FP64 potentials and energy
    density, one with XC_INCREMENTAL_FP32_POTENTIALS (FP32 potentials,
    float-float energy density).  E_xc agrees to 1e-10 Eh (every functional
    family; unrestricted branch included)."""
    import ctypes
    import chinium_gb300 as cg
    from chinium_gb300._lib import check, lib
    Z, xyz = M.h2o()
    r = run_scf(Z, xyz, functional=functional, charge=charge, mult=mult, precision="fp64", max_iter=8)
    g = r.context["grid"]
    ns = 2 if mult != 1 else 1
    xc = cg.ExchangeCorrelation(spin=ns).Read(functional)
    n = r.nbasis
    Ds = r.D if ns == 2 else [r.D[0]]
    P = np.random.default_rng(1).normal(size=(n, n)) * 1e-4  # an SCF-sized step
    D1 = [d + P + P.T for d in Ds]

    def inc(Dl, code):
        Dc = np.ascontiguousarray(np.stack([d.T for d in Dl]))
        V = np.zeros((ns, n, n))
        e = ctypes.c_double()
        check(lib().xc_build_incremental(g._h, xc._h, ctypes.c_void_p(Dc.ctypes.data), ns, code, ctypes.byref(e),
                                         ctypes.c_void_p(V.ctypes.data)))
        return e.value

    e_anchor = inc(Ds, 2)
    e64 = inc(D1, 0)
    assert e_anchor < 0 and e64 < 0  # physical densities
    inc(Ds, 2)
    eff = inc(D1, 16)
    print("%s mult %d: E_xc %.12f  float-float - FP64 %.2e" % (functional, mult, e64, eff - e64))
    assert abs(eff - e64) < 1e-10
