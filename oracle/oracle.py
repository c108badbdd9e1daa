"""ORACLE -- test infrastructure only.

Python side of the CPU FP64 restatement of Chinium's XC build.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this module; the product never does.

It parses the package data tables independently of the product's C++ loader,
restates the reference's grid construction (src/Grid/GridGeneration.cpp),
libint2's contraction normalisation (called through
src/Integral/Normalization.cpp:11-18) and drives the C kernels in
``xc_oracle.c`` / ``xc_oracle_func.c`` through ctypes.

Parity: grid/AO/density/energy/Fock restate the reference; the functionals
restate libxc's published formulas (unpinned -- libxc is absent).
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
DATA = os.path.join(REPO, "chinium_gb300", "data")
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
ANGSTROM2BOHR = 1.8897259886  # src/Macro/Unit.h:1

_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.oracle_energy.restype = ctypes.c_double
        _lib.oracle_functional_point.restype = ctypes.c_double
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


# ----------------------------------------------------------------- data --

def load_lebedev():
    rules = {}
    with open(os.path.join(DATA, "lebedev.txt")) as f:
        lines = f.read().split("\n")
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        i += 1
        if ln.startswith("order"):
            n = int(ln.split()[1])
            arr = np.array([[float(t) for t in lines[i + k].split()] for k in range(n)])
            rules[n] = arr
            i += n
    return rules


def load_grid_recipes(name):
    out = {}
    with open(os.path.join(DATA, "grids", name + ".txt")) as f:
        lines = [ln.strip() for ln in f if ln.strip() and not ln.startswith("#")]
    i = 0
    while i < len(lines):
        t = lines[i].split()
        assert t[0] == "element"
        z, nshells, ngroups = int(t[1]), int(t[2]), int(t[3])
        radial = t[4:]
        groups = [tuple(int(v) for v in lines[i + 1 + k].split()) for k in range(ngroups)]
        out[z] = (nshells, radial, groups)
        i += 1 + ngroups
    return out


def load_basis(name):
    out = {}
    with open(os.path.join(DATA, "basis", name + ".txt")) as f:
        lines = [ln.strip() for ln in f if ln.strip() and not ln.startswith("#")]
    i = 0
    while i < len(lines):
        t = lines[i].split()
        z, nsh = int(t[1]), int(t[2])
        i += 1
        shells = []
        for _ in range(nsh):
            lval, nprim = (int(v) for v in lines[i].split())
            i += 1
            rows = np.array([[float(v) for v in lines[i + k].split()] for k in range(nprim)])
            i += nprim
            shells.append((lval, rows[:, 0].copy(), rows[:, 1].copy()))
        out[z] = shells
    return out


def load_sap():
    with open(os.path.join(DATA, "sap.txt")) as f:
        lines = [ln.split() for ln in f if ln.strip() and not ln.startswith("#")]
    radii = np.array([float(v) for v in lines[0][1:]])
    tables = {int(ln[0]): np.array([float(v) for v in ln[1:]]) for ln in lines[1:]}
    return radii, tables


# ---------------------------------------------------------------- basis --

def dfact(n):
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def normalize_contraction(l, exps, coefs):
    """libint2 Shell::renorm(): primitive factors for x^l e^{-a r^2}, then the
    contracted self-overlap scaled to one (called via
    src/Integral/Normalization.cpp:11-18, copied into NormalizedCoefficients)."""
    sqrt_pi3 = math.pi ** 1.5
    c = np.array(coefs, dtype=np.float64)
    e = np.array(exps, dtype=np.float64)
    two_a = 2 * e
    c = c * np.sqrt(2.0 ** l * two_a ** (l + 1) * np.sqrt(two_a) / (sqrt_pi3 * dfact(2 * l - 1)))
    norm = 0.0
    n = len(e)
    for p in range(n):
        for q in range(p + 1):
            g = e[p] + e[q]
            norm += (1 if p == q else 2) * dfact(2 * l - 1) * sqrt_pi3 * c[p] * c[q] / (2.0 ** l * g ** (l + 1) * math.sqrt(g))
    return c / math.sqrt(norm)


class Basis:
    """Shells in centre order; P shells Cartesian (type 1, x y z), l >= 2 pure
    (type -l, m = -l..l) as in src/Grid/GridAO.cpp:153-178."""

    def __init__(self, Z, xyz_bohr, name):
        table = load_basis(name)
        self.Z = list(Z)
        self.xyz = np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)
        types, nprim, off, centers, exps, coefs, atom_of = [], [], [], [], [], [], []
        for a, z in enumerate(self.Z):
            for lval, e, c in table[z]:
                types.append(0 if lval == 0 else (1 if lval == 1 else -lval))
                nprim.append(len(e))
                off.append(len(exps))
                centers.append(self.xyz[a])
                exps.extend(e)
                coefs.extend(normalize_contraction(lval, e, c))
                atom_of.append(a)
        self.types = np.array(types, dtype=np.int32)
        self.nprim = np.array(nprim, dtype=np.int32)
        self.off = np.array(off, dtype=np.int32)
        self.centers = np.array(centers, dtype=np.float64)
        self.exps = np.array(exps, dtype=np.float64)
        self.coefs = np.array(coefs, dtype=np.float64)
        self.shell_atom = np.array(atom_of, dtype=np.int32)
        self.nbasis = int(sum(1 if t == 0 else (3 if abs(t) == 1 else 2 * abs(t) + 1) for t in types))

    def ao(self, x, y, z, deriv=1):
        ng = len(x)
        ao = np.zeros(self.nbasis * ng)
        ao1 = np.zeros(3 * self.nbasis * ng) if deriv else np.zeros(1)
        lib().oracle_ao(ctypes.c_int(len(self.types)), _p(self.types), _p(self.nprim), _p(self.off),
                        _p(self.centers), _p(self.exps), _p(self.coefs), ctypes.c_int(self.nbasis),
                        ctypes.c_int(ng), _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(y)),
                        _p(np.ascontiguousarray(z)), ctypes.c_int(deriv), _p(ao), _p(ao1))
        return ao.reshape(self.nbasis, ng), (ao1.reshape(3, self.nbasis, ng) if deriv else None)

    def ao2(self, x, y, z):
        """Second derivatives (6, n, g): xx, xy, yy, xz, yz, zz (SubGrid::AO2's packing)."""
        ng = len(x)
        out = np.zeros(6 * self.nbasis * ng)
        lib().oracle_ao2(ctypes.c_int(len(self.types)), _p(self.types), _p(self.nprim), _p(self.off),
                         _p(self.centers), _p(self.exps), _p(self.coefs), ctypes.c_int(self.nbasis),
                         ctypes.c_int(ng), _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(y)),
                         _p(np.ascontiguousarray(z)), _p(out))
        return out.reshape(6, self.nbasis, ng)

    def ao3(self, x, y, z):
        """Third derivatives (10, n, g), the packed sorted triples (xxx, xxy, xyy, yyy, xxz, ...)."""
        ng = len(x)
        out = np.zeros(10 * self.nbasis * ng)
        lib().oracle_ao3(ctypes.c_int(len(self.types)), _p(self.types), _p(self.nprim), _p(self.off),
                         _p(self.centers), _p(self.exps), _p(self.coefs), ctypes.c_int(self.nbasis),
                         ctypes.c_int(ng), _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(y)),
                         _p(np.ascontiguousarray(z)), _p(out))
        return out.reshape(10, self.nbasis, ng)

    def function_atoms(self):
        """Atom of every basis function."""
        out = []
        for t, a in zip(self.types, self.shell_atom):
            out.extend([a] * (1 if t == 0 else (3 if abs(t) == 1 else 2 * abs(t) + 1)))
        return np.array(out, dtype=np.int32)


# ----------------------------------------------------------------- grid --

def atom_points(z, xyz, recipes, lebedev):
    """SphericalGrid (GridGeneration.cpp:73-133) for one atom: coordinates and
    radial * 4 pi * Lebedev weight, in generation order."""
    nshells_total, radial, groups = recipes[z]
    kind = radial[0]
    if kind == "de2":
        a, t2, t3 = float(radial[1]), float(radial[2]), float(radial[3])
        h = (t3 - t2) / float(nshells_total - 1)

        def ri(i):
            xi = h * i + t2
            return math.exp(a * xi - math.exp(-xi))

        def rw(i):
            xi = h * i + t2
            return math.exp(3 * a * xi - 3 * math.exp(-xi)) * (a + math.exp(-xi)) * h
    elif kind == "em":
        R = float(radial[1])

        def ri(i):
            ii = i + 1
            return R * math.pow(ii / (nshells_total + 1 - ii), 2)

        def rw(i):
            ii = i + 1
            return 2 * math.pow(R, 3) * (nshells_total + 1) * math.pow(ii, 5) / math.pow(nshells_total + 1 - ii, 7)
    else:
        raise ValueError("unrecognized radial formula")
    xs, ys, zs, ws = [], [], [], []
    ish = 0
    for npts, nsh in groups:
        rule = lebedev[npts]
        for _ in range(nsh):
            r = ri(ish)
            w_r = rw(ish)
            xs.append(rule[:, 0] * r + xyz[0])
            ys.append(rule[:, 1] * r + xyz[1])
            zs.append(rule[:, 2] * r + xyz[2])
            ws.append(w_r * (4 * math.pi * rule[:, 3]))
            ish += 1
    return np.concatenate(xs), np.concatenate(ys), np.concatenate(zs), np.concatenate(ws)


def grid_points(Z, xyz_bohr, grid_name, return_unpartitioned=False):
    """All points (x, y, z, w) in the reference's generation order with
    Becke-partitioned weights."""
    lebedev = load_lebedev()
    recipes = load_grid_recipes(grid_name)
    xyz = np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)
    parts = [atom_points(z, xyz[a], recipes, lebedev) for a, z in enumerate(Z)]
    owner = np.concatenate([np.full(len(p[0]), a, dtype=np.int32) for a, p in enumerate(parts)])
    px = np.concatenate([p[0] for p in parts])
    py = np.concatenate([p[1] for p in parts])
    pz = np.concatenate([p[2] for p in parts])
    w_in = np.concatenate([p[3] for p in parts])
    w = np.empty_like(w_in)
    lib().oracle_becke(ctypes.c_int(len(Z)), _p(np.ascontiguousarray(xyz.ravel())), ctypes.c_long(len(px)),
                       _p(px), _p(py), _p(pz), _p(owner), _p(w_in), _p(w))
    if return_unpartitioned:
        return px, py, pz, w, w_in
    return px, py, pz, w


def block_ranges(npts, max_size=128):
    """RecursiveCut (GridGeneration.cpp:177-210) as it behaves: the partition
    step touches only the first four points, so leaves are recursive halves
    of generation order (left half = floor(n/2))."""
    out = []

    def rec(lo, n):
        if n <= max_size:
            out.append((lo, n))
        else:
            h = n // 2
            rec(lo, h)
            rec(lo + h, n - h)

    rec(0, npts)
    return out


def padded_blocks(px, py, pz, w):
    """SubGrid::SubGrid (GridGeneration.cpp:212-230): pad to a multiple of 8,
    padded coordinates copy the block's first points, padded weights are 0."""
    blocks = []
    for lo, n in block_ranges(len(px)):
        npad = (n + 7) & ~7
        sl = slice(lo, lo + n)
        bx, by, bz, bw = (np.zeros(npad) for _ in range(4))
        bx[:n], by[:n], bz[:n], bw[:n] = px[sl], py[sl], pz[sl], w[sl]
        extra = npad - n
        bx[n:], by[n:], bz[n:] = bx[:extra], by[:extra], bz[:extra]
        blocks.append((bx, by, bz, bw))
    return blocks


# ------------------------------------------------------------ functionals --

def functional(ids, nspin, rho, sigma=None, tau=None):
    """eps, vrho, vsigma, vtau on points; reference per-block layout
    (rho (s, g), sigma (ns(ns+1)/2, g), tau (s, g))."""
    ids = np.asarray(ids, dtype=np.int32)
    rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(nspin, -1)
    ng = rho.shape[1]
    nsig = 1 if nspin == 1 else 3
    sigma = np.zeros((nsig, ng)) if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(nsig, ng)
    tau = np.zeros((nspin, ng)) if tau is None else np.ascontiguousarray(tau, dtype=np.float64).reshape(nspin, ng)
    eps = np.zeros(ng)
    vrho = np.zeros((nspin, ng))
    vsigma = np.zeros((nsig, ng))
    vtau = np.zeros((nspin, ng))
    st = lib().oracle_functional(ctypes.c_int(len(ids)), _p(ids), ctypes.c_int(nspin), ctypes.c_int(ng),
                                 _p(rho), _p(sigma), _p(tau), _p(eps), _p(vrho), _p(vsigma), _p(vtau))
    if st:
        raise ValueError("unknown functional id in %s" % list(ids))
    return eps, vrho, vsigma, vtau


def functional_fxc(ids, nspin, rho, sigma=None):
    """v2rho2, v2rhosigma, v2sigma2 on points (libxc layouts, component-major);
    LDA and GGA only."""
    ids = np.asarray(ids, dtype=np.int32)
    rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(nspin, -1)
    ng = rho.shape[1]
    nsig, nrr, nrs = (1, 1, 1) if nspin == 1 else (3, 3, 6)
    sigma = np.zeros((nsig, ng)) if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(nsig, ng)
    v2rho2, v2rhosigma, v2sigma2 = np.zeros((nrr, ng)), np.zeros((nrs, ng)), np.zeros((nrs, ng))
    st = lib().oracle_functional_fxc(ctypes.c_int(len(ids)), _p(ids), ctypes.c_int(nspin), ctypes.c_int(ng),
                                     _p(rho), _p(sigma), _p(v2rho2), _p(v2rhosigma), _p(v2sigma2))
    if st:
        raise ValueError("second derivatives need LDA / GGA ids, got %s" % list(ids))
    return v2rho2, v2rhosigma, v2sigma2


def functional_point(ids, nspin, inputs):
    ids = np.asarray(ids, dtype=np.int32)
    x = np.ascontiguousarray(inputs, dtype=np.float64)
    return lib().oracle_functional_point(ctypes.c_int(len(ids)), _p(ids), ctypes.c_int(nspin), _p(x))


FUNCTIONAL_FILES = {  # DensityFunctionals/<name>.df contents (libxc ids)
    "SLATER": [1], "SVWN5": [1, 7], "B88": [106], "BLYP": [106, 131], "B3LYP": [402],
    "BHHLYP": [436], "PBE": [321, 322], "PBE0": [406], "TPSS": [202, 231], "TPSSH": [457],
    "R2SCAN": [497, 498],
}
EXX = {402: 0.20, 406: 0.25, 436: 0.5, 457: 0.10}


def family(ids):
    fam = 0
    for i in ids:
        if i in (101, 106, 130, 131, 321, 322, 402, 406, 436):
            fam = max(fam, 1)
        elif i in (202, 231, 457, 497, 498):
            fam = max(fam, 2)
    return fam


# ------------------------------------------------------------------ build --

class OracleGrid:
    """Grid + per-block AO, mirroring Grid::Grid and Grid::getAO."""

    def __init__(self, basis, grid_name, Z, xyz_bohr, deriv=1):
        self.basis = basis
        px, py, pz, w, w_in = grid_points(Z, xyz_bohr, grid_name, return_unpartitioned=True)
        self.npoints = len(px)
        self.blocks = padded_blocks(px, py, pz, w)
        # radial * 4 pi * Lebedev weight before the Becke factor, padded like w
        self.w_unpartitioned = np.concatenate([b[3] for b in padded_blocks(px, py, pz, w_in)])
        self.deriv = deriv
        self.ao = []
        for bx, by, bz, bw in self.blocks:
            self.ao.append(basis.ao(bx, by, bz, deriv))

    def build(self, D, ids, nspin, nblocks=None, nthreads=0):
        """Density -> functional -> energy -> Fock over the first nblocks
        blocks with the C oracle (OpenMP).  D: (nspin, n, n)."""
        fam = family(ids)
        nb = self.basis.nbasis
        blocks = self.blocks[: nblocks or len(self.blocks)]
        ngs = np.array([len(b[0]) for b in blocks], dtype=np.int32)
        pt_off = np.concatenate([[0], np.cumsum(ngs)[:-1]]).astype(np.int64)
        ao_off = (pt_off * nb).astype(np.int64)
        w = np.concatenate([b[3] for b in blocks])
        ao = np.concatenate([a[0].ravel() for a in self.ao[: len(blocks)]])
        ao1 = np.concatenate([a[1].ravel() for a in self.ao[: len(blocks)]]) if fam >= 1 else np.zeros(1)
        Dc = np.ascontiguousarray(np.asarray(D, dtype=np.float64).reshape(nspin, nb, nb).transpose(0, 2, 1))
        F = np.zeros((nspin, nb, nb))
        E = ctypes.c_double()
        idsa = np.asarray(ids, dtype=np.int32)
        st = lib().oracle_build(ctypes.c_int(len(blocks)), _p(ngs), _p(pt_off), _p(ao_off), _p(w), _p(ao), _p(ao1),
                                ctypes.c_int(nb), ctypes.c_int(nspin), ctypes.c_int(fam), _p(Dc),
                                ctypes.c_int(len(idsa)), _p(idsa), ctypes.c_int(nthreads), ctypes.byref(E), _p(F))
        if st:
            raise ValueError("oracle build failed")
        return E.value, F.transpose(0, 2, 1).copy()


    def build_response(self, D, DU, ids, nspin, nblocks=None, nthreads=0):
        """response() over the first nblocks blocks with the C driver (OpenMP over blocks):
        the timed CPU baseline.  Returns V_U (nspin, nmat, n, n)."""
        fam = family(ids)
        nb = self.basis.nbasis
        blocks = self.blocks[: nblocks or len(self.blocks)]
        ngs = np.array([len(b[0]) for b in blocks], dtype=np.int32)
        pt_off = np.concatenate([[0], np.cumsum(ngs)[:-1]]).astype(np.int64)
        ao_off = (pt_off * nb).astype(np.int64)
        w = np.concatenate([b[3] for b in blocks])
        ao = np.concatenate([a[0].ravel() for a in self.ao[: len(blocks)]])
        ao1 = np.concatenate([a[1].ravel() for a in self.ao[: len(blocks)]]) if fam >= 1 else np.zeros(1)
        D = np.asarray(D, dtype=np.float64).reshape(nspin, nb, nb)
        DU = np.asarray(DU, dtype=np.float64).reshape(nspin, -1, nb, nb)
        nmat = DU.shape[1]
        Dc = np.ascontiguousarray(D.transpose(0, 2, 1))
        DUc = np.ascontiguousarray(DU.transpose(0, 1, 3, 2))
        F = np.zeros((nspin, nmat, nb, nb))
        idsa = np.asarray(ids, dtype=np.int32)
        st = lib().oracle_build_response(ctypes.c_int(len(blocks)), _p(ngs), _p(pt_off), _p(ao_off), _p(w), _p(ao),
                                         _p(ao1), ctypes.c_int(nb), ctypes.c_int(nspin), ctypes.c_int(fam), _p(Dc),
                                         ctypes.c_int(nmat), _p(DUc), ctypes.c_int(len(idsa)), _p(idsa),
                                         ctypes.c_int(nthreads), _p(F))
        if st:
            raise ValueError("oracle response build failed")
        return F.transpose(0, 1, 3, 2).copy()

    def response(self, D, DU, ids, nspin):
        """getDensity(D) + Evaluate("v", "f") + getDensityU(DU) + getFockU<u_t>
        block by block with the C oracle (GridDensity.cpp:47-77,
        GridFock.cpp:97-160).  D (nspin, n, n); DU (nspin, nmat, n, n).
        Returns V_U (nspin, nmat, n, n)."""
        fam = family(ids)
        nb = self.basis.nbasis
        D = np.asarray(D, dtype=np.float64).reshape(nspin, nb, nb)
        DU = np.asarray(DU, dtype=np.float64).reshape(nspin, -1, nb, nb)
        nmat = DU.shape[1]
        Dc = np.ascontiguousarray(D.transpose(0, 2, 1))       # column-major per spin
        DUc = np.ascontiguousarray(DU.transpose(0, 1, 3, 2))  # (mu, nu, mat, s) column-major
        F = np.zeros((nspin, nmat, nb, nb))
        blist = np.arange(nb, dtype=np.int32)
        nsig = 1 if nspin == 1 else 3
        L = lib()
        for b, blk in enumerate(self.blocks):
            ng = len(blk[0])
            w = np.ascontiguousarray(blk[3], dtype=np.float64)
            ao = np.ascontiguousarray(self.ao[b][0], dtype=np.float64)
            ao1 = np.ascontiguousarray(self.ao[b][1], dtype=np.float64) if fam >= 1 else np.zeros(1)
            rho, rho1 = np.zeros(nspin * ng), np.zeros(nspin * 3 * ng)
            sigma, tau = np.zeros(nsig * ng), np.zeros(nspin * ng)
            L.oracle_density(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(nspin), ctypes.c_int(fam), _p(Dc),
                             _p(ao), _p(ao1), _p(rho), _p(rho1), _p(sigma), _p(tau))
            vsigma = functional(ids, nspin, rho, sigma)[2] if fam >= 1 else np.zeros((nsig, ng))
            v2rho2, v2rhosigma, v2sigma2 = functional_fxc(ids, nspin, rho, sigma)
            rhoU, rho1U, sigmaU = np.zeros(nspin * nmat * ng), np.zeros(nspin * nmat * 3 * ng), np.zeros(nsig * nmat * ng)
            L.oracle_density_u(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(nspin), ctypes.c_int(nmat),
                               ctypes.c_int(fam), _p(DUc), _p(ao), _p(ao1), _p(rho1), _p(rhoU), _p(rho1U), _p(sigmaU))
            vsigma = np.ascontiguousarray(vsigma)
            L.oracle_fock_u(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(nb), _p(blist), ctypes.c_int(nspin),
                            ctypes.c_int(nmat), ctypes.c_int(fam), _p(w), _p(ao), _p(ao1), _p(rho1), _p(vsigma),
                            _p(v2rho2), _p(v2rhosigma), _p(v2sigma2), _p(rhoU), _p(rho1U), _p(sigmaU), _p(F))
        return F.transpose(0, 1, 3, 2).copy()


    def fock_skeleton(self, D, ids, nspin):
        """The Hessian's skeleton V_xc derivatives for every atom A and direction t with the grid
        fixed: getFockSkeleton (GridFock.cpp:52-95) and getFockU<s_t> on the skeleton density
        derivatives of getDensitySkeleton (GridDensity.cpp:79-130, GridFock.cpp:97-160), block by
        block.  D (nspin, n, n).  Returns (F_skeleton, F_U) as (nspin, 3 natoms, n, n), matrix
        3 A + t; their sum is dV_xc / dR_(A,t) at fixed D."""
        fam = family(ids)
        nb = self.basis.nbasis
        natoms = len(self.basis.Z)
        D = np.asarray(D, dtype=np.float64).reshape(nspin, nb, nb)
        Dc = np.ascontiguousarray(D.transpose(0, 2, 1))
        nmat = 3 * natoms
        Fs = np.zeros((nspin, natoms, 3, nb, nb))
        Fu = np.zeros((nspin, nmat, nb, nb))
        blist = np.arange(nb, dtype=np.int32)
        atom_of = self.basis.function_atoms()
        nsig = 1 if nspin == 1 else 3
        L = lib()
        for b, blk in enumerate(self.blocks):
            ng = len(blk[0])
            w = np.ascontiguousarray(blk[3], dtype=np.float64)
            ao = np.ascontiguousarray(self.ao[b][0], dtype=np.float64)
            ao1 = np.ascontiguousarray(self.ao[b][1], dtype=np.float64)
            ao2 = np.ascontiguousarray(self.basis.ao2(blk[0], blk[1], blk[2])) if fam >= 1 else np.zeros(1)
            rho, rho1 = np.zeros(nspin * ng), np.zeros(nspin * 3 * ng)
            sigma, tau = np.zeros(nsig * ng), np.zeros(nspin * ng)
            L.oracle_density(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(nspin), ctypes.c_int(fam), _p(Dc),
                             _p(ao), _p(ao1), _p(rho), _p(rho1), _p(sigma), _p(tau))
            _, vrho, vsigma, _ = functional(ids, nspin, rho, sigma)
            vrho, vsigma = np.ascontiguousarray(vrho), np.ascontiguousarray(vsigma)
            v2rho2, v2rhosigma, v2sigma2 = functional_fxc(ids, nspin, rho, sigma)
            rg, r1g, sg = np.zeros(nmat * nspin * ng), np.zeros(3 * nmat * nspin * ng), np.zeros(nmat * nsig * ng)
            L.oracle_density_skeleton(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(nspin), ctypes.c_int(natoms),
                                      _p(atom_of), ctypes.c_int(fam), _p(Dc), _p(ao), _p(ao1), _p(ao2), _p(rho1),
                                      _p(rg), _p(r1g), _p(sg))
            L.oracle_fock_skeleton(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(nb), _p(blist),
                                   ctypes.c_int(nspin), ctypes.c_int(natoms), _p(atom_of), ctypes.c_int(fam), _p(w),
                                   _p(ao), _p(ao1), _p(ao2), _p(rho1), _p(vrho), _p(vsigma), _p(Fs))
            L.oracle_fock_u(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(nb), _p(blist), ctypes.c_int(nspin),
                            ctypes.c_int(nmat), ctypes.c_int(fam), _p(w), _p(ao), _p(ao1), _p(rho1), _p(vsigma),
                            _p(v2rho2), _p(v2rhosigma), _p(v2sigma2), _p(rg), _p(r1g), _p(sg), _p(Fu))
        Fs = Fs.reshape(nspin, nmat, nb, nb).transpose(0, 1, 3, 2).copy()
        return Fs, Fu.transpose(0, 1, 3, 2).copy()


def energy_hess(og, D, ids):
    """XC skeleton energy Hessian with the grid fixed, restricted: getDensitySkeleton2 +
    getEnergyHess (GridDensity.cpp:132-212, GridEnergy.cpp:32-46) block by block.  D the total
    density (n, n).  Returns (3 natoms, 3 natoms), index 3 a + t."""
    fam = family(ids)
    b = og.basis
    nb, natoms = b.nbasis, len(b.Z)
    nm = 3 * natoms
    Dc = np.ascontiguousarray(np.asarray(D, dtype=np.float64).reshape(nb, nb).T)
    atom_of = b.function_atoms()
    E = np.zeros(nm * nm)
    L = lib()
    for k, blk in enumerate(og.blocks):
        ng = len(blk[0])
        w = np.ascontiguousarray(blk[3], dtype=np.float64)
        ao = np.ascontiguousarray(og.ao[k][0])
        ao1 = np.ascontiguousarray(og.ao[k][1])
        ao2 = np.ascontiguousarray(b.ao2(blk[0], blk[1], blk[2]))
        ao3 = np.ascontiguousarray(b.ao3(blk[0], blk[1], blk[2])) if fam >= 1 else np.zeros(1)
        rho, rho1, sigma, tau = np.zeros(ng), np.zeros(3 * ng), np.zeros(ng), np.zeros(ng)
        L.oracle_density(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(1), ctypes.c_int(fam), _p(Dc), _p(ao),
                         _p(ao1), _p(rho), _p(rho1), _p(sigma), _p(tau))
        _, vrho, vsigma, _ = functional(ids, 1, rho, sigma)
        vrho, vsigma = np.ascontiguousarray(vrho), np.ascontiguousarray(vsigma)
        f2 = [np.ascontiguousarray(a) for a in functional_fxc(ids, 1, rho, sigma)]
        rg, r1g, sg = np.zeros(nm * ng), np.zeros(3 * nm * ng), np.zeros(nm * ng)
        L.oracle_density_skeleton(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(1), ctypes.c_int(natoms),
                                  _p(atom_of), ctypes.c_int(fam), _p(Dc), _p(ao), _p(ao1), _p(ao2), _p(rho1), _p(rg),
                                  _p(r1g), _p(sg))
        L.oracle_energy_hess(ctypes.c_int(ng), ctypes.c_int(nb), ctypes.c_int(natoms), _p(atom_of), ctypes.c_int(fam),
                             _p(Dc), _p(w), _p(ao), _p(ao1), _p(ao2), _p(ao3), _p(rho1), _p(vrho), _p(vsigma), _p(f2[0]),
                             _p(f2[1]), _p(f2[2]), _p(rg), _p(r1g), _p(sg), _p(E))
    return E.reshape(nm, nm).T.copy()


def energy_hess_fd(og, Z, xyz_bohr, basis_name, D, ids, pairs, h=1e-3):
    """d^2 E_xc / dR_i dR_j at fixed D with the grid fixed (i, j = 3 atom + direction) for the
    given pairs, by the four-point difference of E_xc with the basis functions of the atoms
    displaced, steps h and h/2 combined by Richardson extrapolation.  Test reference for
    energy_hess."""
    xyz = np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)
    saved = og.ao, og.basis

    def energy(moves):
        moved = xyz.copy()
        for (i, d) in moves:
            moved[i // 3, i % 3] += d
        bm = Basis(Z, moved, basis_name)
        og.basis = bm
        og.ao = [bm.ao(bx, by, bz, og.deriv) for bx, by, bz, bw in og.blocks]
        return og.build(np.asarray(D)[None], ids, 1)[0]

    out = {}
    try:
        for i, j in pairs:
            vals = []
            for hh in (h, 0.5 * h):
                e = [energy([(i, si * hh), (j, sj * hh)]) for si, sj in ((1, 1), (1, -1), (-1, 1), (-1, -1))]
                vals.append((e[0] - e[1] - e[2] + e[3]) / (4 * hh * hh))
            out[(i, j)] = (4 * vals[1] - vals[0]) / 3
    finally:
        og.ao, og.basis = saved
    return out


def fock_fd(og, Z, xyz_bohr, basis_name, D, ids, nspin, h=1e-4):
    """dV_xc / dR_(A,t) at fixed D with the grid held fixed, by central
    differences of the oracle's V_xc with atom A's basis functions displaced
    by +-h and +-h/2 (Richardson); (nspin, 3 natoms, n, n).  Test reference
    for fock_skeleton."""
    xyz = np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)
    saved = og.ao, og.basis
    n = og.basis.nbasis
    out = np.zeros((nspin, 3 * len(Z), n, n))
    try:
        for a in range(len(Z)):
            for t in range(3):
                cds = []
                for hh in (h, 0.5 * h):
                    vs = []
                    for sgn in (1.0, -1.0):
                        moved = xyz.copy()
                        moved[a, t] += sgn * hh
                        bm = Basis(Z, moved, basis_name)
                        og.basis = bm
                        og.ao = [bm.ao(bx, by, bz, og.deriv) for bx, by, bz, bw in og.blocks]
                        vs.append(np.array(og.build(D, ids, nspin)[1]))
                    cds.append((vs[0] - vs[1]) / (2 * hh))
                out[:, 3 * a + t] = (4 * cds[1] - cds[0]) / 3
    finally:
        og.ao, og.basis = saved
    return out


def skeleton_grad_fd(og, Z, xyz_bohr, basis_name, D, ids, nspin, h=1e-4):
    """Nuclear gradient of E_xc with the grid held fixed by central finite
    differences: the basis functions of one atom are displaced by +-h along
    one axis and E_xc is rebuilt on the unchanged grid points at fixed D --
    the quantity SubGrid::getDensitySkeleton + SubGrid::getEnergyGrad give
    analytically (GridDensity.cpp:79-130, GridEnergy.cpp:15-30).  Richardson
    extrapolation of the steps h and h/2 leaves an O(h^4) error (~1e-10 Eh/bohr
    for H2O).  Test infrastructure; (natoms, 3)."""
    g1 = _central_fd(og, Z, xyz_bohr, basis_name, D, ids, nspin, h)
    g2 = _central_fd(og, Z, xyz_bohr, basis_name, D, ids, nspin, 0.5 * h)
    return (4.0 * g2 - g1) / 3.0


def _central_fd(og, Z, xyz_bohr, basis_name, D, ids, nspin, h):
    xyz = np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)
    saved = og.ao, og.basis
    out = np.zeros((len(Z), 3))
    try:
        for a in range(len(Z)):
            for t in range(3):
                es = []
                for sgn in (1.0, -1.0):
                    moved = xyz.copy()
                    moved[a, t] += sgn * h
                    bm = Basis(Z, moved, basis_name)
                    og.basis = bm
                    og.ao = [bm.ao(bx, by, bz, og.deriv) for bx, by, bz, bw in og.blocks]
                    es.append(og.build(D, ids, nspin)[0])
                out[a, t] = (es[0] - es[1]) / (2 * h)
    finally:
        og.ao, og.basis = saved
    return out
