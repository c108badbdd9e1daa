"""GPU parity: the CUDA path through the C ABI against the oracle on the same
inputs.  Tolerances: FP64 path 1e-10 Eh in E_xc and 1e-10 max-abs in V_xc
(the parity bar for the plain path); pointwise stages (weights, AO, densities,
functional) at 1e-12 relative or tighter where FP64 rounding allows."""
import numpy as np
import pytest

import chinium_gb300 as cg
from chinium_gb300 import molecules as M
from conftest import model_density
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL = 1e-10
V_TOL = 1e-10


@pytest.fixture(scope="module")
def h2o(h2o_oracle):
    Z, xyz, ob, og = h2o_oracle
    b = cg.Basis(Z, xyz, "def2-svp")
    return Z, xyz, b, ob, og


def make_grid(b, nspin=1, type_=1, thr=0.0, grid="SG-1"):
    g = cg.Grid(b, grid, nspin=nspin, screen_threshold=thr)
    g.setType(type_)
    g.getAO(0)
    return g


def test_points_and_becke_weights(h2o):
    Z, xyz, b, ob, og = h2o
    g = make_grid(b)
    p = g.points()
    ox = np.concatenate([bl[0] for bl in og.blocks])
    ow = np.concatenate([bl[3] for bl in og.blocks])
    assert g.info()["npoints"] == og.npoints == 11320
    assert g.info()["nblocks"] == 128
    assert np.array_equal(p["x"], ox)
    # Becke factors near cell boundaries come from 1 - p3 with p3 ~ 1, so a
    # weight is only as precise as its unpartitioned radial*angular weight
    rel = np.abs(p["w"] - ow) / np.maximum(og.w_unpartitioned, 1e-300)
    real = og.w_unpartitioned > 0
    assert np.all(p["w"][~real] == 0)
    assert rel[real].max() <= 1e-12, (rel.max(), int(np.argmax(rel)))


def test_ao_values_all_blocks(h2o):
    Z, xyz, b, ob, og = h2o
    g = make_grid(b, type_=1)
    for blk in range(0, 128, 7):
        ao, ao1, lst = g.block_ao(blk)
        oao, oao1 = og.ao[blk]
        assert np.array_equal(lst, np.arange(24))
        assert np.allclose(ao, oao, rtol=1e-13, atol=1e-15)
        assert np.allclose(ao1, oao1, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("type_", [0, 1, 2])
def test_density_values(h2o, type_):
    Z, xyz, b, ob, og = h2o
    D = model_density(og, 5)
    g = make_grid(b, type_=type_)
    g.getDensity([D])
    dv = g.density_values()
    off = 0
    for (bx, by, bz, bw), (ao, ao1) in zip(og.blocks, og.ao):
        ng = len(bx)
        rho = np.einsum("mg,mn,ng->g", ao, D, ao)
        assert np.allclose(dv["rho"][0, off:off + ng], rho, rtol=1e-12, atol=1e-14)
        if type_ >= 1:
            r1 = 2 * np.einsum("rmg,mn,ng->rg", ao1, D, ao)
            assert np.allclose(dv["rho1"][0, :, off:off + ng], r1, rtol=1e-11, atol=1e-13)
        if type_ >= 2:
            tau = 0.5 * np.einsum("rmg,mn,rng->g", ao1, D, ao1)
            assert np.allclose(dv["tau"][0, off:off + ng], tau, rtol=1e-11, atol=1e-13)
        off += ng
    assert g.getNumElectrons() == pytest.approx(10.0, abs=1e-9)


@pytest.mark.parametrize("ids", [[1], [1, 7], [8], [106], [131], [101, 130], [321, 322], [402], [406], [436],
                                 [202, 231], [457], [497, 498]])
@pytest.mark.parametrize("ns", [1, 2])
def test_functional_points(ids, ns):
    rng = np.random.default_rng(7)
    n = 400
    fam = O.family(ids)
    if ns == 1:
        rho = 10 ** rng.uniform(-9, 3, n)
        sig = rho ** (8 / 3) * 10 ** rng.uniform(-4, 1.5, n)
        tau = sig / (8 * rho) * (1 + 10 ** rng.uniform(-4, 1, n))
        rho[:5] = [0, 1e-16, 1e-15, 2e-15, 1e-14]
        args = (rho, sig, tau)
    else:
        ra = 10 ** rng.uniform(-9, 3, n)
        rb = ra * 10 ** rng.uniform(-3, 0.5, n)
        saa = ra ** (8 / 3) * 10 ** rng.uniform(-4, 1.5, n)
        sbb = rb ** (8 / 3) * 10 ** rng.uniform(-4, 1.5, n)
        sab = np.sqrt(saa * sbb) * rng.uniform(-1, 1, n)
        ta = saa / (8 * ra) * (1 + 10 ** rng.uniform(-4, 1, n))
        tb = sbb / (8 * rb) * (1 + 10 ** rng.uniform(-4, 1, n))
        rb[:3] = 0.0  # fully polarised points
        args = (np.stack([ra, rb]), np.stack([saa, sab, sbb]), np.stack([ta, tb]))
    ref = O.functional(ids, ns, *args)
    got = cg.ExchangeCorrelation.from_ids(ids, spin=ns).eval_points(*args)
    # Relative agreement; inputs span 12 decades and reach the density
    # threshold, where the functional's own conditioning amplifies ulp
    # differences of pow/exp/log between the device and host libraries.
    # Bar: 1e-9 for 99% of points (PBE-type correlation goes through
    # exp(x) - 1 at small |eps_c|, which loses digits in both codes) and 1e-8
    # everywhere a spin density is >= 1e-12; points with a spin density below
    # that (at the threshold, carrying <= 1e-12 electrons per unit volume)
    # agree to 1e-3.
    names = ["eps", "vrho", "vsigma", "vtau"]
    dens = args[0].reshape(ns, n)
    low = (dens < 1e-12).any(axis=0)
    for k, (r, q) in enumerate(zip(ref, got)):
        if k == 2 and fam < 1 or k == 3 and fam < 2:
            continue
        assert np.all(np.isfinite(q))
        scale = np.abs(r).max() + 1e-300
        err = (np.abs(q - r) / (np.abs(r) + 1e-14 * scale)).reshape(-1, n)
        assert np.quantile(err, 0.99) < 1e-9, (names[k], np.quantile(err, 0.99))
        assert err[:, ~low].max() < 1e-8, (names[k], err[:, ~low].max())
        assert err[:, low].max(initial=0) < 1e-3, (names[k], err[:, low].max(initial=0))


CASES = [("PBE", 1, [321, 322]), ("B3LYP", 1, [402]), ("SVWN5", 0, [1, 7]), ("TPSS", 2, [202, 231]),
         ("R2SCAN", 2, [497, 498])]


@pytest.mark.parametrize("name,type_,ids", CASES)
def test_exc_vxc_restricted(h2o, name, type_, ids):
    Z, xyz, b, ob, og = h2o
    D = model_density(og, 5)
    xc = cg.ExchangeCorrelation().Read(name)
    g = make_grid(b, type_=type_)
    E, V = g.build(xc, [D])
    Eo, Fo = og.build([D], ids, 1)
    assert abs(E - Eo) <= E_TOL, (E, Eo)
    assert np.abs(V[0] - Fo[0]).max() <= V_TOL
    # split entry points agree with the fused call
    g.getDensity([D])
    xc.Evaluate("ev", g)
    assert g.getEnergy() == pytest.approx(E, abs=1e-13)
    assert np.abs(g.getFock()[0] - V[0]).max() < 1e-13


@pytest.mark.parametrize("name,type_,ids", [("PBE", 1, [321, 322]), ("TPSS", 2, [202, 231]), ("B3LYP", 1, [402])])
def test_exc_vxc_unrestricted(h2o, name, type_, ids):
    Z, xyz, b, ob, og = h2o
    Da, Db = model_density(og, (5, 4), nspin=2, seed=2)
    xc = cg.ExchangeCorrelation(spin=2).Read(name)
    g = make_grid(b, nspin=2, type_=type_)
    E, V = g.build(xc, [Da, Db])
    Eo, Fo = og.build([Da, Db], ids, 2)
    assert abs(E - Eo) <= E_TOL
    for s in range(2):
        assert np.abs(V[s] - Fo[s]).max() <= V_TOL


def test_screening_is_exact_to_threshold(h2o):
    Z, xyz, b, ob, og = h2o
    D = model_density(og, 5)
    xc = cg.ExchangeCorrelation().Read("B3LYP")
    E0, V0 = make_grid(b, thr=0.0).build(xc, [D])
    g = make_grid(b, thr=1e-15)
    E1, V1 = g.build(xc, [D])
    assert g.info()["screened_pairs"] <= 128 * 24 * 24
    assert abs(E1 - E0) < 1e-12
    assert np.abs(V1[0] - V0[0]).max() < 1e-12


def test_energy_is_deterministic(h2o):
    Z, xyz, b, ob, og = h2o
    D = model_density(og, 5)
    xc = cg.ExchangeCorrelation().Read("PBE")
    g = make_grid(b)
    E1, V1 = g.build(xc, [D])
    E2, V2 = g.build(xc, [D])
    assert E1 == E2
    assert np.abs(V1[0] - V2[0]).max() < 1e-14


def test_sap_fock(h2o):
    Z, xyz, b, ob, og = h2o
    g = make_grid(b, type_=0)
    V = g.sap_fock()
    radii, tables = O.load_sap()
    tab = np.stack([tables[z] for z in Z])
    import ctypes
    F = np.zeros((24, 24))
    for (bx, by, bz, bw), (ao, _) in zip(og.blocks, og.ao):
        v = np.zeros(len(bx))
        O.lib().oracle_sap(ctypes.c_int(3), O._p(np.ascontiguousarray(xyz.ravel())), O._p(np.ascontiguousarray(tab)),
                           O._p(radii), ctypes.c_int(751), ctypes.c_long(len(bx)), O._p(bx), O._p(by), O._p(bz), O._p(v))
        F += (ao * (bw * v)) @ ao.T
    assert np.abs(V - F).max() < 1e-10


MIXED_E_TOL = 1e-5   # Eh, split-BF16 (~FP32) contractions with FP64 accumulation
MIXED_V_TOL = 1e-5


@pytest.mark.parametrize("name,type_,nspin", [("SVWN5", 0, 1), ("PBE", 1, 1), ("B3LYP", 1, 1), ("TPSS", 2, 1),
                                              ("R2SCAN", 2, 1), ("PBE", 1, 2), ("TPSS", 2, 2)])
def test_mixed_precision_against_fp64(h2o, name, type_, nspin):
    """Tensor-core path vs the FP64 path on the same grid and density."""
    Z, xyz, b, ob, og = h2o
    if nspin == 1:
        D = [model_density(og, 5)]
    else:
        D = list(model_density(og, (5, 4), nspin=2, seed=2))
    xc = cg.ExchangeCorrelation(spin=nspin).Read(name)
    g = make_grid(b, nspin=nspin, type_=type_)
    E64, V64 = g.build(xc, D)
    E32, V32 = g.build(xc, D, precision=cg.PRECISION_MIXED)
    dE = abs(E32 - E64)
    dV = max(np.abs(V32[s] - V64[s]).max() for s in range(nspin))
    print("mixed vs fp64 %s ns=%d: |dE|=%.3e max|dV|=%.3e" % (name, nspin, dE, dV))
    assert dE < MIXED_E_TOL and dV < MIXED_V_TOL, (dE, dV)
    for s in range(nspin):
        assert np.allclose(V32[s], V32[s].T, atol=1e-14)
    # a second call reuses the prepared tiles and gives the same result
    E32b, V32b = g.build(xc, D, precision=cg.PRECISION_MIXED)
    assert E32b == E32


def test_sap_fock_tensor_cores(h2o):
    """The tensor-core SAP matrix against the FP64 one (FP32-level accuracy)."""
    Z, xyz, b, ob, og = h2o
    g = make_grid(b, type_=0)
    V64 = g.sap_fock()
    Vtc = g.sap_fock(cg.PRECISION_MIXED)
    scale = np.abs(V64).max()
    print("SAP tensor-core vs FP64: max|dV| %.2e of max|V| %.2e" % (np.abs(Vtc - V64).max(), scale))
    assert np.abs(Vtc - V64).max() < 2e-6 * scale
    assert np.allclose(Vtc, Vtc.T, atol=1e-14)


@pytest.mark.parametrize("name,type_,nspin", [("SVWN5", 0, 1), ("PBE", 1, 1), ("PBE", 1, 2), ("B3LYP", 1, 1)])
def test_xc_gradient_against_oracle_finite_differences(h2o, name, type_, nspin):
    """dE_xc/dR with the grid fixed (getDensitySkeleton + getEnergyGrad): the
    CUDA FP64 gradient against central finite differences of the oracle's
    E_xc with one atom's basis functions displaced (Richardson-extrapolated
    steps of 1e-4 and 5e-5 bohr, accurate to ~1e-9)."""
    Z, xyz, b, ob, og = h2o
    xc = cg.ExchangeCorrelation(spin=nspin).Read(name)
    g = cg.Grid(b, "SG-1", nspin=nspin)
    g.setType(type_)
    g.getAO(1)
    D = [model_density(og, 5)] if nspin == 1 else model_density(og, (5, 4), nspin=2, seed=2)
    G = g.getEnergyGrad(xc, D)
    ref = O.skeleton_grad_fd(og, Z, xyz, "def2-svp", np.stack(D), O.FUNCTIONAL_FILES[name], nspin)
    print(name, nspin, "max |dG| %.2e, max |G| %.2e" % (np.abs(G - ref).max(), np.abs(ref).max()))
    assert np.abs(G - ref).max() < 1e-8
    # the gradient needs the AO derivatives one order above the functional's
    g0 = make_grid(b, nspin=nspin, type_=type_)
    with pytest.raises(cg.XCError):
        g0.getEnergyGrad(xc, D)


def test_xc_gradient_rejects_meta_gga(h2o):
    """The reference's skeleton gradient has no tau terms; neither has this one."""
    Z, xyz, b, ob, og = h2o
    xc = cg.ExchangeCorrelation().Read("TPSS")
    g = make_grid(b, type_=2)
    with pytest.raises(cg.XCError) as e:
        g.getEnergyGrad(xc, [model_density(og, 5)])
    assert e.value.code == -6


def test_grid_from_caller_shells_is_bitwise_the_named_basis(h2o):
    """xc_basis_create_shells with the shells of the named basis (normalised
    coefficients, as the Mwfn's NormalizedCoefficients): bitwise the same
    E_xc and V_xc equal to rounding (FP64 atomics), FP64 and tensor-core paths."""
    Z, xyz, b, ob, og = h2o
    sh = b.shells()
    b2 = cg.Basis.from_shells(Z, xyz, sh["atom"], sh["type"], sh["nprim"], sh["exps"], sh["coefs"])
    D = model_density(og, 5)
    xc = cg.ExchangeCorrelation().Read("PBE")
    for prec in (cg.PRECISION_FP64, cg.PRECISION_MIXED):
        E1, V1 = make_grid(b).build(xc, [D], precision=prec)
        E2, V2 = make_grid(b2).build(xc, [D], precision=prec)
        assert E1 == E2  # E_xc is summed in a fixed order
        assert np.abs(V1[0] - V2[0]).max() < 1e-14  # V_xc takes FP64 atomics: equal to rounding
