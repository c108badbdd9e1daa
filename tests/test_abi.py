"""CPU tests of the C ABI and host logic (no GPU computation)."""
import ctypes
import subprocess

import numpy as np
import pytest

import chinium_gb300 as cg
from chinium_gb300 import molecules as M
from chinium_gb300._lib import LIB_PATH, header_symbols, lib
from conftest import has_gpu
from oracle import oracle as O


def test_library_exports_every_header_symbol():
    L = lib()
    syms = header_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(L, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(syms) <= exported


@pytest.mark.parametrize("mol,basis,n", [("h2o", "def2-svp", 24), ("c18", "def2-tzvp", 558), ("fe4s4", "def2-tzvp", 328)])
def test_basis_sizes(mol, basis, n):
    Z, xyz = getattr(M, mol)()
    assert cg.Basis(Z, xyz, basis).nbasis == n


def test_basis_normalisation_matches_oracle():
    Z, xyz = M.fe4s4()
    b = cg.Basis(Z, xyz, "def2-tzvp")
    ob = O.Basis(Z, xyz, "def2-tzvp")
    sh = b.shells()
    assert np.array_equal(sh["type"], ob.types)
    assert np.array_equal(sh["nprim"], ob.nprim)
    assert np.allclose(sh["exps"], ob.exps, rtol=0, atol=0)
    assert np.allclose(sh["coefs"], ob.coefs, rtol=1e-14)


def test_alkane_batch_shapes():
    mols = M.alkane_batch(64, seed=0)
    assert len(mols) == 64
    for Z, xyz in mols:
        nC = Z.count(6)
        assert Z.count(1) == 2 * nC + 2
        d = np.linalg.norm(xyz[:, None] - xyz[None], axis=-1) + np.eye(len(Z)) * 10
        assert d.min() > 0.9 * M.ANGSTROM2BOHR


def test_c18_and_fe4s4_geometry():
    Z, xyz = M.c18()
    r = np.linalg.norm(xyz, axis=1) / M.ANGSTROM2BOHR
    assert np.allclose(r, 3.88)
    d = np.linalg.norm(np.roll(xyz, -1, 0) - xyz, axis=1) / M.ANGSTROM2BOHR
    assert np.allclose(d[0::2] / d[1::2], 1.22 / 1.35)
    Z, xyz = M.fe4s4()
    dfs = [np.linalg.norm(xyz[i] - xyz[j]) / M.ANGSTROM2BOHR for i in range(4) for j in range(4, 8)]
    assert sorted(dfs)[:12] == pytest.approx([2.28] * 12, abs=1e-9)


def test_integrals_structure():
    """S, T, V against grid quadrature on the oracle grid; ERI symmetry and
    positive semidefiniteness of the (mu nu | lambda sigma) supermatrix."""
    from chinium_gb300.scf import one_electron, repulsion
    from oracle import oracle as O
    Z, xyz = M.h2o()
    b = cg.Basis(Z, xyz, "def2-svp")
    S, T, V = one_electron(b)
    assert np.allclose(np.diag(S), 1.0, atol=1e-12)
    assert np.allclose(S, S.T) and np.allclose(T, T.T) and np.allclose(V, V.T)
    og = O.OracleGrid(O.Basis(Z, xyz, "def2-svp"), "SG-1", Z, xyz)
    Sg, Tg, Vg = (np.zeros_like(S) for _ in range(3))
    for (bx, by, bz, bw), (ao, ao1) in zip(og.blocks, og.ao):
        Sg += (ao * bw) @ ao.T
        Tg += 0.5 * sum((ao1[r] * bw) @ ao1[r].T for r in range(3))
        vn = sum(-z / np.maximum(np.sqrt((bx - xyz[a, 0]) ** 2 + (by - xyz[a, 1]) ** 2 + (bz - xyz[a, 2]) ** 2), 1e-12)
                 for a, z in enumerate(Z))
        Vg += (ao * (bw * vn)) @ ao.T
    assert np.abs(S - Sg).max() < 1e-4
    assert np.abs(T - Tg).max() < 1e-3
    assert np.abs(V - Vg).max() < 1e-3
    eri = repulsion(b)
    n = b.nbasis
    assert np.allclose(eri, eri.transpose(1, 0, 2, 3)) and np.allclose(eri, eri.transpose(2, 3, 0, 1))
    assert np.linalg.eigvalsh(eri.reshape(n * n, n * n)).min() > -1e-12


def test_functional_read_fields():
    for name, ids, exx, fam in [("PBE", [321, 322], 0.0, "GGA"), ("B3LYP", [402], 0.2, "GGA"),
                                ("TPSS", [202, 231], 0.0, "mGGA"), ("R2SCAN", [497, 498], 0.0, "mGGA"),
                                ("SVWN5", [1, 7], 0.0, "LDA"), ("TPSSH", [457], 0.1, "mGGA")]:
        xc = cg.ExchangeCorrelation().Read(name)
        assert xc.EXX == pytest.approx(exx)
        assert xc.Family == fam
        assert bool(xc)


def test_error_codes():
    with pytest.raises(cg.XCError) as e:
        cg.ExchangeCorrelation().Read("NO_SUCH_FUNCTIONAL")
    assert e.value.code == -2
    with pytest.raises(cg.XCError) as e:
        cg.ExchangeCorrelation().Read("M06-2X")  # ids present in the data, functional not implemented
    assert e.value.code == -6
    with pytest.raises(cg.XCError) as e:
        cg.ExchangeCorrelation.from_ids([402], spin=3)
    assert e.value.code == -1
    with pytest.raises(cg.XCError) as e:
        cg.Basis([8, 1, 1], np.zeros((3, 3)), "no-such-basis")
    assert e.value.code == -2
    with pytest.raises(cg.XCError) as e:
        cg.Basis([54], np.zeros((1, 3)), "def2-svp")  # element outside the packaged tables
    assert e.value.code == -2
    Z, xyz = M.fe4s4()
    b = cg.Basis(Z, xyz, "def2-tzvp")
    with pytest.raises(cg.XCError) as e:
        cg.Grid(b, "SG-1")  # SG-1 has no Fe recipe (the reference throws the same)
    assert e.value.code in (-2, -3)
    buf = ctypes.create_string_buffer(8)
    assert lib().xc_last_error(buf, 8) == 0


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU error path")
def test_grid_without_gpu_fails_loudly():
    Z, xyz = M.h2o()
    b = cg.Basis(Z, xyz, "def2-svp")
    with pytest.raises(cg.XCError) as e:
        cg.Grid(b, "SG-1")
    assert e.value.code == -3


def test_batch_and_tuning_argument_errors():
    """Argument checks of the batch / tuning entry points run before any
    device work (a missing GPU is not reached)."""
    L = lib()
    h = ctypes.c_void_p()
    assert L.xc_grid_create_batch(0, None, b"SG-1", 1, ctypes.byref(h)) == -1
    assert L.xc_grid_create_batch(2, None, b"SG-1", 1, ctypes.byref(h)) == -1
    Z, xyz = M.h2o()
    b = cg.Basis(Z, xyz, "def2-svp")
    arr = (ctypes.c_void_p * 2)(b._h.value, None)
    assert L.xc_grid_create_batch(2, arr, b"SG-1", 1, ctypes.byref(h)) == -1
    arr = (ctypes.c_void_p * 1)(b._h.value)
    assert L.xc_grid_create_batch(1, arr, b"SG-1", 3, ctypes.byref(h)) == -1
    assert L.xc_grid_set_mixed_config(None, None) == -1
    assert L.xc_grid_tune(None, None, None, 1, 1e-7, 1e-6, 1, None) == -1


def test_mixed_config_struct_layout():
    from chinium_gb300._lib import MixedConfig, TuneCandidate, TuneReport
    assert ctypes.sizeof(MixedConfig) == 32
    assert MixedConfig.func_float_above.offset == 16
    assert MixedConfig.v_operands.offset == 24
    assert ctypes.sizeof(TuneCandidate) == 32 + 3 * 8 + 8 + 8
    assert TuneReport.cand.offset == 32 + 8 + 8 + 8


def test_dipole_integrals_shift_symmetry_and_quadrature():
    """xc_dipole: <mu| r - C |nu> = <mu| r |nu> - C S exactly, symmetric, and
    equal to the SG-3 quadrature of (r - C) phi phi within that quadrature's
    own error on S."""
    from chinium_gb300 import molecules as M
    from chinium_gb300.cpscf import dipole_integrals
    from chinium_gb300.scf import one_electron
    from oracle import oracle as O
    Z, xyz = M.h2o()
    b = cg.Basis(Z, xyz, "def2-svp")
    S = one_electron(b)[0]
    C = np.array([0.1, -0.2, 0.3])
    M0, MC = dipole_integrals(b), dipole_integrals(b, C)
    assert np.abs(MC - (M0 - C[:, None, None] * S)).max() < 1e-14
    assert np.array_equal(M0, M0.transpose(0, 2, 1))
    ob = O.Basis(Z, xyz, "def2-svp")
    px, py, pz, w = O.grid_points(Z, xyz, "SG-3")
    n = b.nbasis
    qS, qM = np.zeros((n, n)), np.zeros((3, n, n))
    for i0 in range(0, len(px), 20000):
        sl = slice(i0, i0 + 20000)
        ao = ob.ao(px[sl], py[sl], pz[sl], 0)[0]
        qS += (ao * w[sl]) @ ao.T
        for k, q in enumerate((px[sl], py[sl], pz[sl])):
            qM[k] += (ao * (w[sl] * q)) @ ao.T
    errS = np.abs(S - qS).max()
    assert errS < 5e-5
    assert np.abs(M0 - qM).max() < 5 * errS


def test_response_entry_points_validate_arguments_on_the_host():
    """The response entry points reject null handles and buffers, and meta-GGA
    second derivatives, before touching a device."""
    import ctypes
    from chinium_gb300._lib import lib
    L = lib()
    nul = ctypes.c_void_p()
    one = np.zeros(4)
    p = one.ctypes.data_as(ctypes.c_void_p)
    assert L.xc_grid_get_density_u(nul, p, 1, 1) == -1
    assert L.xc_grid_get_fock_u(nul, p) == -1
    assert L.xc_grid_set_response_precision(nul, 0) == -1
    assert L.xc_build_response(nul, nul, p, 1, 0, 1, p, p) == -1
    assert L.xc_functional_fxc_points(nul, 1, p, p, p, p, p) == -1
    assert L.xc_dipole(nul, p, p) == -1
    assert L.xc_grid_fock_skeleton(nul, nul, p, 1, p, p) == -1
    f = ctypes.c_void_p()
    ids = (ctypes.c_int * 2)(202, 231)
    assert L.xc_functional_create(ids, 2, 1, ctypes.byref(f)) == 0
    try:
        assert L.xc_functional_fxc_points(f, 1, p, p, p, p, p) == -6  # TPSS: no "f" (as the reference)
    finally:
        L.xc_functional_destroy(f)


@pytest.mark.parametrize("mol,basis", [("h2o", "def2-svp"), ("c18", "def2-tzvp"), ("fe4s4", "def2-tzvp")])
def test_basis_from_caller_shells_equals_named_basis(mol, basis):
    """xc_basis_create_shells on the shells a named basis exports (its
    normalised coefficients, as the Mwfn's NormalizedCoefficients) gives the
    same basis; with raw contraction coefficients and normalize=1 the
    libint2 renormalisation reproduces the normalised ones."""
    Z, xyz = getattr(M, mol)()
    b = cg.Basis(Z, xyz, basis)
    sh = b.shells()
    b2 = cg.Basis.from_shells(Z, xyz, sh["atom"], sh["type"], sh["nprim"], sh["exps"], sh["coefs"])
    assert b2.nbasis == b.nbasis
    sh2 = b2.shells()
    for k in ("atom", "type", "first", "nprim", "exps", "coefs"):
        assert np.array_equal(sh2[k], sh[k]), k
    # raw coefficients from the basis table, renormalised by the library
    table = O.load_basis(basis)
    raw = np.concatenate([c for z in Z for (_, _, c) in table[z]])
    b3 = cg.Basis.from_shells(Z, xyz, sh["atom"], sh["type"], sh["nprim"], sh["exps"], raw, normalize=True)
    assert np.allclose(b3.shells()["coefs"], sh["coefs"], rtol=1e-14, atol=0)


def test_basis_from_shells_validates_arguments():
    Z, xyz = M.h2o()
    L = lib()
    h = ctypes.c_void_p()
    Zi = np.array(Z, dtype=np.int32)
    X = np.ascontiguousarray(xyz, dtype=np.float64)
    atom = np.array([0, 7], dtype=np.int32)
    typ = np.array([0, 0], dtype=np.int32)
    npr = np.array([1, 1], dtype=np.int32)
    e = np.array([1.0, 2.0])
    c = np.array([1.0, 1.0])
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    # atom index out of range
    assert L.xc_basis_create_shells(3, p(Zi), p(X), 2, p(atom), p(typ), p(npr), p(e), p(c), 0, ctypes.byref(h)) == -1
    atom[1] = 1
    # Cartesian d (type 2) is not a shell type the reference's grid evaluates
    typ[1] = 2
    assert L.xc_basis_create_shells(3, p(Zi), p(X), 2, p(atom), p(typ), p(npr), p(e), p(c), 0, ctypes.byref(h)) == -6
    typ[1] = -1  # pure p (y, z, x) is
    e[1] = -2.0
    assert L.xc_basis_create_shells(3, p(Zi), p(X), 2, p(atom), p(typ), p(npr), p(e), p(c), 0, ctypes.byref(h)) == -7
    e[1] = 2.0
    assert L.xc_basis_create_shells(3, p(Zi), p(X), 2, p(atom), p(typ), p(npr), p(e), p(c), 2, ctypes.byref(h)) == -1
    assert L.xc_basis_create_shells(3, p(Zi), p(X), 2, p(atom), p(typ), p(npr), p(e), p(c), 1, None) == -1
    assert L.xc_basis_create_shells(3, p(Zi), p(X), 2, p(atom), p(typ), p(npr), p(e), p(c), 1, ctypes.byref(h)) == 0
    n = ctypes.c_int()
    assert L.xc_basis_nbasis(h, ctypes.byref(n)) == 0 and n.value == 4
    L.xc_basis_destroy(h)


def test_static_entry_point_validates_arguments_on_the_host():
    """xc_functional_energy_static rejects bad arguments before touching the
    GPU: null pointers, npoints <= 0, a GGA or meta-GGA call without its
    sigma / tau arrays, and calls above its fixed scratch of 2 097 152 points
    (the pointers below are never dereferenced)."""
    L = lib()
    one = ctypes.c_void_p(16)
    pbe = cg.ExchangeCorrelation().Read("PBE")
    tpss = cg.ExchangeCorrelation().Read("TPSS")
    args = lambda f, n, sig=one, tau=one: (f._h, n, one, one, sig, tau, one, one, sig, tau, one, None)
    msg = lambda: (lambda b: (L.xc_last_error(b, 512), b.value)[1])(ctypes.create_string_buffer(512))
    assert L.xc_functional_energy_static(*args(pbe, 2097152 + 1)) == -1
    assert b"static scratch limit" in msg()
    assert L.xc_functional_energy_static(*args(pbe, 0)) == -1
    assert L.xc_functional_energy_static(*args(pbe, -5)) == -1
    assert L.xc_functional_energy_static(None, 10, one, one, one, one, one, one, one, one, one, None) == -1
    assert L.xc_functional_energy_static(pbe._h, 10, None, one, one, one, one, one, one, one, one, None) == -1
    assert L.xc_functional_energy_static(pbe._h, 10, one, one, one, one, one, one, one, one, None, None) == -1
    assert L.xc_functional_energy_static(*args(pbe, 10, sig=None)) == -1
    assert b"sigma" in msg()
    assert L.xc_functional_energy_static(*args(tpss, 10, tau=None)) == -1
    assert b"tau" in msg()


def test_wait_probe_validates_arguments_on_the_host():
    L = lib()
    assert L.xc_grid_wait_probe(None, 1.0) == -1
