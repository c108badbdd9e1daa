"""Python mirror of the reference's XC interface over the C ABI.

``Grid`` mirrors ``Grid`` (src/Grid/Grid.h:90-116) and ``ExchangeCorrelation``
mirrors ``ExchangeCorrelation`` (src/ExchangeCorrelation.h:8-17): same member
names, argument meaning and call order, so SCF code written against the
reference reads the same:

    grid = Grid(basis, "SG-1", nspin=1); xc = ExchangeCorrelation(); xc.Read("PBE")
    grid.setType(xc.type); grid.getAO(0)
    grid.getDensity([2 * D]); xc.Evaluate("ev", grid)
    Exc = grid.getEnergy(); Vxc = grid.getFock()[0]

Matrices are numpy float64 (n, n); errors raise ``XCError`` (status code +
message), where the reference throws std::runtime_error or asserts.
"""
import ctypes

import numpy as np

from ._lib import GridInfo, MixedConfig, PRECISION_FP64, PRECISION_MIXED, TuneReport, XCError, check, lib

__all__ = ["Basis", "Grid", "BatchGrid", "ExchangeCorrelation", "XCError", "PRECISION_FP64", "PRECISION_MIXED"]


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


class Basis:
    """Centres plus libint2-normalised contracted shells for a named basis
    set (the Mwfn basis after Normalize(), Representation.cpp:30-53), or,
    through ``Basis.from_shells``, the caller's own shells."""

    def __init__(self, Z, xyz_bohr, name):
        Z, xyz = self._centres(Z, xyz_bohr)
        self.Z, self.xyz, self.name = Z, xyz, name
        h = ctypes.c_void_p()
        check(lib().xc_basis_create(len(Z), _p(Z), _p(xyz), name.encode(), ctypes.byref(h)))
        self._adopt(h)

    @staticmethod
    def _centres(Z, xyz_bohr):
        Z = np.ascontiguousarray(Z, dtype=np.int32)
        xyz = np.ascontiguousarray(np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3))
        if len(Z) != len(xyz):
            raise ValueError("Z and coordinates differ in length")
        return Z, xyz

    def _adopt(self, h):
        self._h = h
        n = ctypes.c_int()
        check(lib().xc_basis_nbasis(h, ctypes.byref(n)))
        self.nbasis = n.value

    @classmethod
    def from_shells(cls, Z, xyz_bohr, atom, type, nprim, exps, coefs, normalize=False):
        """The caller's shells (the Mwfn's centres and shells): per shell its
        atom, type (0 s, 1 Cartesian p, -l pure) and primitive count, with
        exps / coefs shell by shell; coefs normalised by the caller
        (NormalizedCoefficients) unless normalize=True."""
        self = cls.__new__(cls)
        Z, xyz = cls._centres(Z, xyz_bohr)
        self.Z, self.xyz, self.name = Z, xyz, None
        atom = np.ascontiguousarray(atom, dtype=np.int32)
        typ = np.ascontiguousarray(type, dtype=np.int32)
        npr = np.ascontiguousarray(nprim, dtype=np.int32)
        e = np.ascontiguousarray(exps, dtype=np.float64)
        c = np.ascontiguousarray(coefs, dtype=np.float64)
        if not (len(atom) == len(typ) == len(npr)) or len(e) != int(npr.sum()) or len(c) != len(e):
            raise ValueError("shell arrays differ in length")
        h = ctypes.c_void_p()
        check(lib().xc_basis_create_shells(len(Z), _p(Z), _p(xyz), len(atom), _p(atom), _p(typ), _p(npr), _p(e),
                                           _p(c), int(bool(normalize)), ctypes.byref(h)))
        self._adopt(h)
        return self

    def shells(self):
        L = lib()
        ns = ctypes.c_int()
        check(L.xc_basis_nshells(self._h, ctypes.byref(ns)))
        atom, typ, first, nprim = (np.zeros(ns.value, dtype=np.int32) for _ in range(4))
        check(L.xc_basis_shells(self._h, _p(atom), _p(typ), _p(first), _p(nprim)))
        exps = np.zeros(int(nprim.sum()))
        coefs = np.zeros(int(nprim.sum()))
        check(L.xc_basis_primitives(self._h, _p(exps), _p(coefs)))
        return dict(atom=atom, type=typ, first=first, nprim=nprim, exps=exps, coefs=coefs)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xc_basis_destroy(h)
            self._h = None


class Grid:
    """Grid::Grid(Mwfn*, grid, nthreads, output) on the GPU.

    screen_threshold: AO magnitude below which a shell is dropped from a block
    (0 keeps every shell in every block, as the reference does)."""

    def __init__(self, basis, grid="SG-1", nspin=1, screen_threshold=0.0):
        self.basis = basis
        self.nspin = nspin
        h = ctypes.c_void_p()
        check(lib().xc_grid_create(basis._h, grid.encode(), nspin, float(screen_threshold), ctypes.byref(h)))
        self._h = h
        self.nbasis = basis.nbasis
        self._nmat_u = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xc_grid_destroy(h)
            self._h = None

    # -- reference members ------------------------------------------------
    def setType(self, type_):
        check(lib().xc_grid_set_type(self._h, int(type_)))

    def getAO(self, derivative=0, output=0):
        check(lib().xc_grid_get_ao(self._h, int(derivative)))

    def getDensity(self, D):
        D = self._stack(D)
        check(lib().xc_grid_get_density(self._h, _p(D), self.nspin))

    def getNumElectrons(self):
        n = ctypes.c_double()
        check(lib().xc_grid_num_electrons(self._h, ctypes.byref(n)))
        return n.value

    def getEnergy(self):
        e = ctypes.c_double()
        check(lib().xc_grid_get_energy(self._h, ctypes.byref(e)))
        return e.value

    def getFock(self):
        n = self.nbasis
        V = np.zeros((self.nspin, n, n))  # column-major per spin == transposed row-major
        check(lib().xc_grid_get_fock(self._h, _p(V)))
        return [V[s].T.copy() for s in range(self.nspin)]

    # -- fused build --------------------------------------------------------
    def build(self, xc, D, precision=PRECISION_FP64):
        """getDensity + Evaluate("ev") + getEnergy + getFock in one call."""
        D = self._stack(D)
        n = self.nbasis
        V = np.zeros((self.nspin, n, n))
        e = ctypes.c_double()
        check(lib().xc_build(self._h, xc._h, _p(D), self.nspin, int(precision), ctypes.byref(e), _p(V)))
        return e.value, [V[s].T.copy() for s in range(self.nspin)]

    def build_device(self, xc, d_D, d_E, d_V, precision=PRECISION_FP64):
        """Device-pointer variant (ints or torch tensors); no synchronisation."""
        ptr = lambda t: ctypes.c_void_p(t if isinstance(t, int) else t.data_ptr())
        check(lib().xc_build_device(self._h, xc._h, ptr(d_D), self.nspin, int(precision), ptr(d_E), ptr(d_V)))

    def wait_probe(self, budget_ms=2.0):
        """Diagnostic: a tensor-core wait that runs out (xc_grid_wait_probe);
        raises XCError with XC_ERR_TIMEOUT."""
        check(lib().xc_grid_wait_probe(self._h, float(budget_ms)))

    def profile(self, enable=True):
        check(lib().xc_grid_profile(self._h, int(bool(enable))))

    # -- mixed-path knobs and autotuner ------------------------------------------
    def mixed_config(self):
        c = MixedConfig()
        check(lib().xc_grid_get_mixed_config(self._h, ctypes.byref(c)))
        return dict(screen=c.screen, fock_tiles=c.fock_tiles, spatial=c.spatial, func_float_above=c.func_float_above,
                    v_operands=c.v_operands)

    def set_mixed_config(self, screen=1e-11, fock_tiles=0, spatial=1, func_float_above=1e-5, v_operands=0):
        """func_float_above: total density from which the mixed path's
        functional runs in FP32 (float("inf"): FP64 everywhere).  v_operands:
        V kernel operands split in-kernel (1), pre-split in HBM (2), or
        chosen by free memory (0)."""
        c = MixedConfig(float(screen), int(fock_tiles), int(spatial), float(func_float_above), int(v_operands), 0)
        check(lib().xc_grid_set_mixed_config(self._h, ctypes.byref(c)))

    def tune(self, xc, D, e_tol=1e-7, v_tol=1e-6, reps=3):
        """Autotune the mixed path on a representative density; the chosen
        configuration stays set.  Returns the tuner's report as a dict."""
        D = self._pack(D)
        r = TuneReport()
        check(lib().xc_grid_tune(self._h, xc._h, _p(D), self.nspin, float(e_tol), float(v_tol), int(reps),
                                 ctypes.byref(r)))
        cfg = lambda c: dict(screen=c.screen, fock_tiles=c.fock_tiles, spatial=c.spatial,
                             func_float_above=c.func_float_above, v_operands=c.v_operands)
        cands = [dict(cfg(c.cfg), ms=c.ms, max_de=c.max_de, max_dv=c.max_dv, kept_pairs=c.kept_pairs,
                      accepted=bool(c.accepted)) for c in r.cand[:r.ncand]]
        return dict(best=cfg(r.best), ms_best=r.ms_best, ms_reference=r.ms_reference, candidates=cands)

    def _pack(self, D):
        return self._stack(D)

    def stage_ms(self):
        """[density, functional, energy, fock] device milliseconds of the last build."""
        ms = np.zeros(4)
        check(lib().xc_grid_stage_ms(self._h, _p(ms)))
        return ms

    def set_stream(self, stream_ptr):
        check(lib().xc_grid_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def kernel_ms(self):
        """[density, functional, energy, Z operand, V partials, V reduction] (ms)
        of the last profiled mixed build."""
        ms = np.zeros(6)
        check(lib().xc_grid_kernel_ms(self._h, _p(ms)))
        return ms

    def getEnergyGrad(self, xc, D):
        """Nuclear gradient of E_xc with the grid fixed (SubGrid::getDensitySkeleton
        + getEnergyGrad); (natoms, 3).  Needs getAO(1) (AO derivatives one
        order above the functional's)."""
        Dst = self._stack(D)
        g = np.zeros(3 * len(self.basis.Z))
        check(lib().xc_grid_energy_grad(self._h, xc._h, _p(Dst), self.nspin, _p(g)))
        return g.reshape(-1, 3)

    # -- response (coupled-perturbed) V_xc ---------------------------------
    def _stack_u(self, DU):
        """DU[spin][mat] (or, for one spin, a list of matrices) -> column-major (s, nmat, n, n)."""
        if self.nspin == 1 and len(DU) and np.asarray(DU[0]).ndim == 2:
            DU = [DU]
        if len(DU) != self.nspin:
            raise XCError(-1, "Wrong number of spin types!")
        nmat = len(DU[0])
        out = np.stack([np.stack([np.asarray(d, dtype=np.float64).T for d in DU[s]]) for s in range(self.nspin)])
        return np.ascontiguousarray(out), nmat

    def _unstack_u(self, F, nmat):
        return [[F[s, m].T.copy() for m in range(nmat)] for s in range(self.nspin)]

    def setResponsePrecision(self, precision):
        """Precision of getDensityU / getFockU (PRECISION_FP64 default;
        PRECISION_MIXED: tensor-core response densities and V_U on the FP64
        ground state of Evaluate("ev") / Evaluate("f"))."""
        check(lib().xc_grid_set_response_precision(self._h, int(precision)))

    def getDensityU(self, DU):
        """Grid::getDensityU: DU[spin][mat] (restricted: a list of matrices)."""
        Du, nmat = self._stack_u(DU)
        check(lib().xc_grid_get_density_u(self._h, _p(Du), self.nspin, nmat))
        self._nmat_u = nmat

    def getFockU(self):
        """Grid::getFockU<u_t>: V_U[spin][mat] of the last getDensityU."""
        n, nmat = self.nbasis, self._nmat_u
        F = np.zeros((self.nspin, nmat, n, n))
        check(lib().xc_grid_get_fock_u(self._h, _p(F)))
        return self._unstack_u(F, nmat)

    def build_response(self, xc, D, DU, precision=PRECISION_FP64):
        """getDensity(D) + Evaluate("ev") + Evaluate("f") + getDensityU(DU) +
        getFockU<u_t> in one call; returns V_U[spin][mat].  PRECISION_MIXED
        forms the response densities and V_U on the tensor cores (symmetric
        part of each D_U)."""
        Dst = self._stack(D)
        Du, nmat = self._stack_u(DU)
        n = self.nbasis
        F = np.zeros((self.nspin, nmat, n, n))
        check(lib().xc_build_response(self._h, xc._h, _p(Dst), self.nspin, int(precision), nmat, _p(Du), _p(F)))
        return self._unstack_u(F, nmat)

    def getFockSkeleton(self, xc, D):
        """getFockSkeleton and getFockU<s_t> (grid fixed, FP64, LDA / GGA) for every atom and
        direction: (FS, FU), each (nspin, 3 natoms, n, n) with matrix 3 A + t; FS + FU is
        dV_xc / dR at fixed D.  Needs getAO(1)."""
        Dst = self._stack(D)
        n, na = self.nbasis, len(self.basis.Z)
        FS = np.zeros((self.nspin, 3 * na, n, n))
        FU = np.zeros((self.nspin, 3 * na, n, n))
        check(lib().xc_grid_fock_skeleton(self._h, xc._h, _p(Dst), self.nspin, _p(FS), _p(FU)))
        return FS.transpose(0, 1, 3, 2).copy(), FU.transpose(0, 1, 3, 2).copy()

    def sap_fock(self, precision=PRECISION_FP64):
        """SuperpositionAtomicPotential (GuessSCF.cpp:17-75); PRECISION_MIXED
        assembles it on the tensor cores (FP32-level accuracy)."""
        n = self.nbasis
        V = np.zeros((n, n))
        fn = lib().xc_sap_fock_tc if precision == PRECISION_MIXED else lib().xc_sap_fock
        check(fn(self._h, _p(V)))
        return V.T.copy()

    # -- inspection -----------------------------------------------------------
    def info(self):
        i = GridInfo()
        check(lib().xc_grid_info_get(self._h, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in GridInfo._fields_}

    def points(self):
        inf = self.info()
        G, nb = inf["npoints_padded"], inf["nblocks"]
        x, y, z, w = (np.zeros(G) for _ in range(4))
        off, ng, nreal, nbas = (np.zeros(nb, dtype=np.int32) for _ in range(4))
        check(lib().xc_grid_points(self._h, _p(x), _p(y), _p(z), _p(w), _p(off), _p(ng), _p(nreal), _p(nbas)))
        return dict(x=x, y=y, z=z, w=w, off=off, ng=ng, nreal=nreal, nb=nbas)

    def density_values(self):
        inf = self.info()
        G, s = inf["npoints_padded"], self.nspin
        rho = np.zeros((s, G))
        rho1 = np.zeros((s, 3, G))
        sigma = np.zeros((1 if s == 1 else 3, G))
        tau = np.zeros((s, G))
        check(lib().xc_grid_density_values(self._h, _p(rho), _p(rho1), _p(sigma), _p(tau)))
        return dict(rho=rho, rho1=rho1, sigma=sigma, tau=tau)

    def potential_values(self):
        inf = self.info()
        G, s = inf["npoints_padded"], self.nspin
        eps = np.zeros(G)
        vrho = np.zeros((s, G))
        vsigma = np.zeros((1 if s == 1 else 3, G))
        vtau = np.zeros((s, G))
        check(lib().xc_grid_potential_values(self._h, _p(eps), _p(vrho), _p(vsigma), _p(vtau)))
        return dict(eps=eps, vrho=vrho, vsigma=vsigma, vtau=vtau)

    def block_ao(self, b):
        p = self.points()
        ng, nb = int(p["ng"][b]), int(p["nb"][b])
        ao = np.zeros((nb, ng))
        ao1 = np.zeros((3, nb, ng))
        lst = np.zeros(nb, dtype=np.int32)
        check(lib().xc_grid_block_ao(self._h, int(b), _p(ao), _p(ao1), _p(lst)))
        return ao, ao1, lst

    def _stack(self, D):
        if isinstance(D, np.ndarray) and D.ndim == 2:
            D = [D]
        D = [np.asarray(d, dtype=np.float64) for d in D]
        if len(D) != self.nspin:
            raise XCError(-1, "Wrong number of spin types!")
        # column-major per spin: store D^T row-major
        return np.ascontiguousarray(np.stack([d.T for d in D]))


class BatchGrid(Grid):
    """Many molecules on one GPU: each keeps its own Becke-partitioned grid
    (as Grid(basis, grid, nspin) with screen threshold 0); the mixed-precision
    build runs the point tiles of all of them in one persistent launch per
    stage, replayed from a CUDA graph.  Mixed precision only.

    D and V are lists over molecules of what Grid.build takes and returns
    (a list of nspin n_m x n_m matrices); E is an array over molecules."""

    def __init__(self, bases, grid="SG-2", nspin=1):
        self.bases = list(bases)
        self.basis = None
        self.nspin = nspin
        arr = (ctypes.c_void_p * len(self.bases))(*[b._h.value for b in self.bases])
        h = ctypes.c_void_p()
        check(lib().xc_grid_create_batch(len(self.bases), arr, grid.encode(), nspin, ctypes.byref(h)))
        self._h = h
        self.nmol = len(self.bases)
        self.nbasis_list = [b.nbasis for b in self.bases]
        self.npoints = np.zeros(self.nmol, dtype=np.int64)
        self.offsets = np.zeros(self.nmol, dtype=np.int64)
        check(lib().xc_grid_molecules(self._h, None, None, _p(self.npoints), _p(self.offsets)))
        self.packed_size = int(sum(nspin * n * n for n in self.nbasis_list))

    def _pack(self, Ds):
        if len(Ds) != self.nmol:
            raise XCError(-1, "one density per molecule")
        out = np.empty(self.packed_size)
        for m, D in enumerate(Ds):
            blk = self._stack(D).ravel()
            o = int(self.offsets[m])
            out[o:o + blk.size] = blk
        return out

    def _unpack(self, V):
        res = []
        for m, n in enumerate(self.nbasis_list):
            o = int(self.offsets[m])
            blk = V[o:o + self.nspin * n * n].reshape(self.nspin, n, n)
            res.append([blk[s].T.copy() for s in range(self.nspin)])
        return res

    def build(self, xc, Ds, precision=PRECISION_MIXED):
        D = self._pack(Ds)
        V = np.zeros(self.packed_size)
        E = np.zeros(self.nmol)
        check(lib().xc_build(self._h, xc._h, _p(D), self.nspin, int(precision), _p(E), _p(V)))
        return E, self._unpack(V)


class ExchangeCorrelation:
    """ExchangeCorrelation (src/ExchangeCorrelation.h:8-17)."""

    def __init__(self, spin=1):
        self.Spin = spin
        self.Codes = []
        self.EXX = 1.0
        self.Family = ""
        self._h = None

    def Read(self, df, output=False):
        h = ctypes.c_void_p()
        check(lib().xc_functional_read(df.encode(), self.Spin, ctypes.byref(h)))
        self._adopt(h)
        return self

    @classmethod
    def from_ids(cls, ids, spin=1):
        self = cls(spin)
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        h = ctypes.c_void_p()
        check(lib().xc_functional_create(_p(ids), len(ids), spin, ctypes.byref(h)))
        self._adopt(h)
        self.Codes = [int(i) for i in ids]
        return self

    def _adopt(self, h):
        if self._h:
            lib().xc_functional_destroy(self._h)
        self._h = h
        e = ctypes.c_double()
        check(lib().xc_functional_exx(h, ctypes.byref(e)))
        f = ctypes.c_int()
        check(lib().xc_functional_family(h, ctypes.byref(f)))
        self.EXX = e.value
        self.type = f.value
        self.Family = ["LDA", "GGA", "mGGA"][f.value]

    def Evaluate(self, order, grid):
        check(lib().xc_evaluate(self._h, grid._h, order.encode()))

    def eval_points(self, rho, sigma=None, tau=None):
        """Pointwise evaluation on host arrays (reference per-point layout)."""
        s = self.Spin
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(s, -1)
        n = rho.shape[1]
        nsig = 1 if s == 1 else 3
        sigma = np.zeros((nsig, n)) if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(nsig, n)
        tau = np.zeros((s, n)) if tau is None else np.ascontiguousarray(tau, dtype=np.float64).reshape(s, n)
        eps = np.zeros(n)
        vrho = np.zeros((s, n))
        vsigma = np.zeros((nsig, n))
        vtau = np.zeros((s, n))
        check(lib().xc_functional_eval_points(self._h, n, _p(rho), _p(sigma), _p(tau), _p(eps), _p(vrho),
                                              _p(vsigma), _p(vtau)))
        return eps, vrho, vsigma, vtau

    def fxc_points(self, rho, sigma=None):
        """Second derivatives (order "f") on host arrays: v2rho2, v2rhosigma,
        v2sigma2 in libxc's layouts, (1 or 3, n), (1 or 6, n), (1 or 6, n)."""
        s = self.Spin
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(s, -1)
        n = rho.shape[1]
        nsig, nrr, nrs = (1, 1, 1) if s == 1 else (3, 3, 6)
        sigma = np.zeros((nsig, n)) if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(nsig, n)
        v2rho2, v2rhosigma, v2sigma2 = np.zeros((nrr, n)), np.zeros((nrs, n)), np.zeros((nrs, n))
        check(lib().xc_functional_fxc_points(self._h, n, _p(rho), _p(sigma), _p(v2rho2), _p(v2rhosigma),
                                             _p(v2sigma2)))
        return v2rho2, v2rhosigma, v2sigma2

    def __bool__(self):
        return self._h is not None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xc_functional_destroy(h)
            self._h = None
