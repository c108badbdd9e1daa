"""GPU parity at the benchmark configurations: the plain FP64 CUDA path
through the C ABI against the oracle on the whole grid, same geometry, basis,
functional, grid and density.  Bar: 1e-10 Eh in E_xc and 1e-10 max-abs in
V_xc (the plain path's parity bar), AO values and gradients to 1e-12
relative (these configurations carry f shells, reference GridAO.cpp:153-178
with AO/PureF.hpp:1-7, and Fe's eight-primitive s shell).

  - cyclo[18]carbon, RKS B3LYP / def2-TZVP (558 functions), SG-2
  - Fe4S4 cubane, UKS TPSS / def2-TZVP (328 functions), multiplicity 9, SG-3
  - one alkane of the 64-alkane batch (seed 0), RKS r2SCAN / def2-SVP, SG-2

The oracle runs with OpenMP over blocks (a few seconds to half a minute per
configuration on the host cores)."""
import numpy as np
import pytest

import chinium_gb300 as cg
from chinium_gb300 import molecules as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL = 1e-10
V_TOL = 1e-10


def orthonormal_density(n, nocc, seed):
    """C C^T of nocc orthonormal columns mixed onto a diagonal occupation
    profile: symmetric, positive semidefinite (rho >= 0), SCF-shaped."""
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(n, nocc)) * 0.05
    A[np.arange(nocc), np.arange(nocc)] += 1.0
    Q, _ = np.linalg.qr(A)
    return Q @ Q.T


def one_alkane():
    """The first molecule of the seed-0 batch with 6..10 carbons."""
    for Z, xyz in M.alkane_batch(64, seed=0):
        if 6 <= Z.count(6) <= 10:
            return Z, xyz
    raise AssertionError("no alkane of 6..10 carbons in the batch")


CONFIGS = {
    "c18": dict(mol=M.c18, basis="def2-tzvp", grid="SG-2", functional="B3LYP", nspin=1, type_=1),
    "fe4s4": dict(mol=M.fe4s4, basis="def2-tzvp", grid="SG-3", functional="TPSS", nspin=2, type_=2,
                  nocc=(88, 80)),
    "alkane": dict(mol=one_alkane, basis="def2-svp", grid="SG-2", functional="R2SCAN", nspin=1, type_=2),
}


@pytest.fixture(scope="module", params=sorted(CONFIGS))
def config(request):
    c = CONFIGS[request.param]
    Z, xyz = c["mol"]()
    ob = O.Basis(Z, xyz, c["basis"])
    og = O.OracleGrid(ob, c["grid"], Z, xyz)
    b = cg.Basis(Z, xyz, c["basis"])
    assert b.nbasis == ob.nbasis
    n = b.nbasis
    if c["nspin"] == 1:
        D = [2.0 * orthonormal_density(n, sum(Z) // 2, seed=3)]
    else:
        D = [orthonormal_density(n, k, seed=4 + s) for s, k in enumerate(c["nocc"])]
    return dict(c, name=request.param, Z=Z, xyz=xyz, ob=ob, og=og, b=b, D=D)


def test_block_structure_matches_oracle(config):
    g = cg.Grid(config["b"], config["grid"], nspin=config["nspin"])
    info = g.info()
    og = config["og"]
    assert info["npoints"] == og.npoints
    assert info["nblocks"] == len(og.blocks)
    p = g.points()
    # coordinates r * (Lebedev direction) + centre: the host compilers may
    # contract the multiply-add (Arm) or not, so equal to a few ulps
    for k, ax in enumerate("xyz"):
        ref = np.concatenate([bl[k] for bl in og.blocks])
        assert np.all(np.abs(p[ax] - ref) <= 1e-14 * np.maximum(np.abs(ref), 1.0)), ax
    assert np.array_equal(p["ng"], [len(bl[0]) for bl in og.blocks])


def test_ao_values_with_f_shells(config):
    """AO values and gradients of every function, f shells included, on blocks
    spread over the grid (near nuclei, bond regions and outer shells)."""
    g = cg.Grid(config["b"], config["grid"], nspin=config["nspin"])
    g.setType(1)
    g.getAO(0)
    og = config["og"]
    types = config["ob"].types
    if config["basis"] == "def2-tzvp":
        assert (types == -3).any(), "def2-TZVP without f shells"
    nblk = len(og.blocks)
    for blk in sorted(set(np.linspace(0, nblk - 1, 24).astype(int))):
        ao, ao1, lst = g.block_ao(int(blk))
        oao, oao1 = og.ao[blk]
        assert np.array_equal(lst, np.arange(config["b"].nbasis))
        scale = np.abs(oao).max() + 1e-300
        assert np.abs(ao - oao).max() <= 1e-12 * scale, (blk, np.abs(ao - oao).max(), scale)
        scale1 = np.abs(oao1).max() + 1e-300
        assert np.abs(ao1 - oao1).max() <= 1e-12 * scale1, (blk, np.abs(ao1 - oao1).max(), scale1)


def test_fp64_build_matches_oracle(config):
    """E_xc and V_xc of the whole grid: CUDA FP64 vs the oracle, 1e-10."""
    c = config
    ids = O.FUNCTIONAL_FILES[c["functional"]]
    xc = cg.ExchangeCorrelation(spin=c["nspin"]).Read(c["functional"])
    g = cg.Grid(c["b"], c["grid"], nspin=c["nspin"])
    g.setType(xc.type)
    assert xc.type == c["type_"]
    g.getAO(0)
    E, V = g.build(xc, c["D"])
    Eo, Fo = c["og"].build(c["D"], ids, c["nspin"])
    dV = max(float(np.abs(V[s] - Fo[s]).max()) for s in range(c["nspin"]))
    print("%s FP64 vs oracle: E_xc %.12f |dE| %.2e max|dV| %.2e (max|V| %.2e)" % (
        c["name"], E, abs(E - Eo), dV, max(float(np.abs(f).max()) for f in Fo)))
    assert abs(E - Eo) <= E_TOL, (E, Eo)
    assert dV <= V_TOL
    # electron count of the density on the grid
    ne = sum(float(np.sum(d * _grid_overlap_trace_weights(c))) for d in c["D"])
    assert g.getNumElectrons() == pytest.approx(ne, rel=1e-12)


def _grid_overlap_trace_weights(c):
    """The grid overlap S_grid = sum_g w phi phi^T (so that N = tr(D S_grid))."""
    if "_S" not in c:
        n = c["b"].nbasis
        S = np.zeros((n, n))
        for (bx, by, bz, bw), (ao, _) in zip(c["og"].blocks, c["og"].ao):
            S += (ao * bw) @ ao.T
        c["_S"] = S
    return c["_S"]


def test_grid_from_caller_shells_is_bitwise_the_named_basis(config):
    """A grid built from the caller's shells (xc_basis_create_shells, the
    Mwfn-shell form of Grid::Grid) gives bitwise the same E_xc and V_xc as
    the grid of the named basis, on the shells that basis exports (V_xc to
    rounding: its FP64 sums use atomics)."""
    if config["name"] != "c18":
        pytest.skip("one large configuration suffices (H2O in test_gpu_parity.py)")
    c = config
    sh = c["b"].shells()
    b2 = cg.Basis.from_shells(c["Z"], c["xyz"], sh["atom"], sh["type"], sh["nprim"], sh["exps"], sh["coefs"])
    xc = cg.ExchangeCorrelation(spin=c["nspin"]).Read(c["functional"])
    out = []
    for b in (c["b"], b2):
        g = cg.Grid(b, c["grid"], nspin=c["nspin"])
        g.setType(xc.type)
        g.getAO(0)
        out.append(g.build(xc, c["D"]))
    assert out[0][0] == out[1][0]  # E_xc is summed in a fixed order
    # V_xc takes FP64 atomics: equal to rounding
    assert all(np.abs(a - b).max() < 1e-13 for a, b in zip(out[0][1], out[1][1]))
