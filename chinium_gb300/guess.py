"""Learned starting density: a per-atom-pair MLP over local geometry.

For every atom pair (A, B) -- including A = B -- a local frame is built from
the pair axis (or, on site, the nearest neighbour) and a reference atom.  The
network sees rotation-invariant features (element types, the pair distance,
and the neighbours' coordinates in that frame) and predicts the density
matrix block D[A, B] expressed in the frame; the block is rotated back to
the molecular frame with the real-solid-harmonic rotation matrices of each
shell.  The assembled matrix is made symmetric and purified to an idempotent
closed-shell density with the right electron count (natural orbitals in the
overlap metric).  Molecules the model does not cover (other elements, other
basis) fall back to the SAP guess.

Training data are converged densities from this library's own SCF; the
network is trained and evaluated by the library's CUDA kernels
(include/chinium_guess.h).
"""
import ctypes
import math
import os

import numpy as np

from ._lib import check, lib

ELEMENTS = (1, 8)          # H, O: the water-cluster model
MAX_FUNC = 14              # def2-SVP: O 14 functions, H 5
N_NEIGH = 12
CUTOFF = 12.0              # bohr
NIN = 7 + 6 * N_NEIGH
NOUT = MAX_FUNC * MAX_FUNC
HIDDEN, LAYERS = 256, 3


# ----------------------------------------------------------------- rotations

def _binom(n, k):
    return math.comb(n, k) if 0 <= k <= n else 0


_SH_TABLES = {}


def _solid_harmonic_table(l):
    """Monomial exponents (a, b, c), a + b + c = l, and the (2l+1) x nmono
    coefficients of the real solid harmonics S_lm (m = -l..l) in them,
    Helgaker-Jorgensen-Olsen normalisation (S_l0 = r^l P_l(cos theta))."""
    if l not in _SH_TABLES:
        exps = [(a, b, l - a - b) for a in range(l, -1, -1) for b in range(l - a, -1, -1)]
        col = {e: i for i, e in enumerate(exps)}
        T = np.zeros((2 * l + 1, len(exps)))
        for m in range(-l, l + 1):
            am = abs(m)
            vm2 = 1 if m < 0 else 0
            N = 1.0 / (2 ** am * math.factorial(l)) * math.sqrt(
                2.0 * math.factorial(l + am) * math.factorial(l - am) / (2.0 if m == 0 else 1.0))
            vmax2 = 2 * math.floor(am / 2 - vm2 / 2) + vm2
            for t in range((l - am) // 2 + 1):
                for u in range(t + 1):
                    for v2 in range(vm2, vmax2 + 1, 2):
                        sgn = -1.0 if (t + (v2 - vm2) // 2) % 2 else 1.0
                        C = sgn * 0.25 ** t * _binom(l, t) * _binom(l - t, am + t) * _binom(t, u) * _binom(am, v2)
                        a, b, c = 2 * t + am - 2 * u - v2, 2 * u + v2, l - 2 * t - am
                        if a < 0 or b < 0 or c < 0:
                            continue
                        T[m + l, col[(a, b, c)]] += N * C
        _SH_TABLES[l] = (exps, T)
    return _SH_TABLES[l]


def solid_harmonics(l, xyz):
    """Real solid harmonics S_lm (m = -l..l), Helgaker-Jorgensen-Olsen
    normalisation (S_l0 = r^l P_l(cos theta)); xyz (K, 3) -> (2l+1, K)."""
    exps, T = _solid_harmonic_table(l)
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    px = [np.ones_like(x)]
    py, pz = [np.ones_like(y)], [np.ones_like(z)]
    for _ in range(l):
        px.append(px[-1] * x)
        py.append(py[-1] * y)
        pz.append(pz[-1] * z)
    mono = np.stack([px[a] * py[b] * pz[c] for a, b, c in exps])
    return T @ mono


_RNG_PTS = np.random.default_rng(12345).normal(size=(32, 3))
_BPINV = {}


def _sample_pinv(l):
    if l not in _BPINV:
        _BPINV[l] = np.linalg.pinv(solid_harmonics(l, _RNG_PTS))
    return _BPINV[l]


def shell_rotations(shell_type, Qs):
    """U_p with f_local = U_p f_global for the functions of one shell, for
    frames Qs (P, 3, 3) whose columns are the local axes in global
    coordinates: S(Q^T r) = U S(r), fitted on 32 sample points."""
    P = len(Qs)
    if shell_type == 0:
        return np.ones((P, 1, 1))
    if shell_type == 1:  # Cartesian x, y, z
        return np.ascontiguousarray(np.transpose(Qs, (0, 2, 1)))
    l = -shell_type
    pts = np.matmul(_RNG_PTS, Qs).reshape(-1, 3)  # rows r^T Q
    A = solid_harmonics(l, pts).reshape(2 * l + 1, P, len(_RNG_PTS)).transpose(1, 0, 2)
    return A @ _sample_pinv(l)


def atom_rotations(shell_types, Qs):
    """Block-diagonal rotation of all functions of one atom, (P, n, n)."""
    blocks = [shell_rotations(t, Qs) for t in shell_types]
    n = sum(b.shape[1] for b in blocks)
    U = np.zeros((len(Qs), n, n))
    o = 0
    for b in blocks:
        k = b.shape[1]
        U[:, o:o + k, o:o + k] = b
        o += k
    return U


def shell_rotation(shell_type, Q):
    return shell_rotations(shell_type, Q[None])[0]


def atom_rotation(shell_types, Q):
    return atom_rotations(shell_types, Q[None])[0]


# -------------------------------------------------------------- geometry

def _frame(ez, ref):
    ez = ez / np.linalg.norm(ez)
    v = ref - np.dot(ref, ez) * ez
    if np.linalg.norm(v) < 1e-6:
        alt = np.array([1.0, 0.0, 0.0]) if abs(ez[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
        v = alt - np.dot(alt, ez) * ez
    ex = v / np.linalg.norm(v)
    ey = np.cross(ez, ex)
    return np.stack([ex, ey, ez], axis=1)


def _by_distance(d, exclude):
    """Atom indices by distance; distances equal to 1e-6 bohr (symmetric
    neighbours, e.g. the two hydrogens of a water) tie-break by index, so the
    order does not depend on rounding or on the molecule's orientation."""
    order = np.lexsort((np.arange(len(d)), np.round(d, 6)))
    return [int(i) for i in order if i not in exclude]


def pair_frame(xyz, a, b):
    """Local axes (columns) for pair (a, b): z along a->b (on site: toward the
    nearest neighbour), x toward the nearest other atom."""
    ra = xyz[a]
    d = np.linalg.norm(xyz - ra, axis=1)
    order = _by_distance(d, (a, b))
    if a == b:
        if len(order) < 1:
            return np.eye(3)
        ez = xyz[order[0]] - ra
        ref = xyz[order[1]] - ra if len(order) > 1 else np.array([1.0, 0.0, 0.0])
    else:
        ez = xyz[b] - ra
        ref = xyz[order[0]] - ra if order else np.array([1.0, 0.0, 0.0])
    return _frame(ez, ref)


def _cut(r):
    return np.where(r < CUTOFF, 0.5 * (np.cos(np.pi * r / CUTOFF) + 1.0), 0.0)


def pair_features(Z, xyz, a, b, Q):
    onehot = lambda z: [1.0 if z == e else 0.0 for e in ELEMENTS]
    dab = np.linalg.norm(xyz[b] - xyz[a])
    f = onehot(Z[a]) + onehot(Z[b]) + [1.0 if a == b else 0.0, dab, math.exp(-dab)]
    ra = xyz[a]
    d = np.linalg.norm(xyz - ra, axis=1)
    order = _by_distance(d, (a, b))[:N_NEIGH]
    for i in order:
        loc = Q.T @ (xyz[i] - ra)
        w = _cut(d[i])
        f += list(loc * w) + [w / (1.0 + d[i])] + onehot(Z[i])
    f += [0.0] * (6 * (N_NEIGH - len(order)))
    return np.array(f, dtype=np.float32)


def frames_and_features(Z, xyz, pr):
    """pair_frame and pair_features for every pair at once: frames (P, 3, 3)
    and features (P, NIN), identical to the per-pair functions."""
    xyz = np.asarray(xyz, dtype=np.float64)
    Z = np.asarray(Z)
    n = len(xyz)
    dist = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=2)
    # per atom, all atoms by distance (ties within 1e-6 bohr by index), as _by_distance
    orders = np.lexsort((np.broadcast_to(np.arange(n), (n, n)), np.round(dist, 6)), axis=-1)
    P = len(pr)
    prs = np.asarray(pr, dtype=np.int64).reshape(P, 2)
    A, B = prs[:, 0], prs[:, 1]
    # the first N_NEIGH + 2 atoms of a's order other than a and b (-1 when the molecule has fewer)
    O = orders[A]
    keep = (O != A[:, None]) & (O != B[:, None])
    sel = np.argsort(~keep, axis=1, kind="stable")[:, :N_NEIGH + 2]
    neigh = np.where(np.take_along_axis(keep, sel, 1), np.take_along_axis(O, sel, 1), -1)
    if neigh.shape[1] < N_NEIGH + 2:
        neigh = np.pad(neigh, ((0, 0), (0, N_NEIGH + 2 - neigh.shape[1])), constant_values=-1)
    ra = xyz[A]
    same = A == B
    # frame: z along a->b (on site: toward the nearest neighbour), x toward the next reference atom
    ez = np.where(same[:, None], xyz[np.maximum(neigh[:, 0], 0)] - ra, xyz[B] - ra)
    ref_idx = np.where(same, neigh[:, 1], neigh[:, 0])
    ref = np.where((ref_idx >= 0)[:, None], xyz[np.maximum(ref_idx, 0)] - ra, np.array([1.0, 0.0, 0.0]))
    lone = same & (neigh[:, 0] < 0)
    ez = ez / np.linalg.norm(np.where(lone[:, None], 1.0, ez), axis=1, keepdims=True)
    v = ref - np.sum(ref * ez, axis=1, keepdims=True) * ez
    alt = np.where((np.abs(ez[:, 0]) < 0.9)[:, None], np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0]))
    valt = alt - np.sum(alt * ez, axis=1, keepdims=True) * ez
    v = np.where((np.linalg.norm(v, axis=1) < 1e-6)[:, None], valt, v)
    ex = v / np.linalg.norm(v, axis=1, keepdims=True)
    ey = np.cross(ez, ex)
    Qs = np.stack([ex, ey, ez], axis=2)
    Qs[lone] = np.eye(3)
    # features
    oh = lambda zz: np.stack([(zz == e).astype(np.float64) for e in ELEMENTS], axis=1)
    dab = dist[A, B]
    cols = [oh(Z[A]), oh(Z[B]), same[:, None].astype(np.float64), dab[:, None], np.exp(-dab)[:, None]]
    # the N_NEIGH nearest others, all at once: (local position x cutoff weight, weight / (1 + d), element)
    ii = neigh[:, :N_NEIGH]
    ok = (ii >= 0)[:, :, None]
    iic = np.maximum(ii, 0)
    di = dist[A[:, None], iic]
    w = _cut(di)
    loc = np.matmul(xyz[iic] - ra[:, None, :], Qs) * w[:, :, None]
    ohk = np.stack([(Z[iic] == e).astype(np.float64) for e in ELEMENTS], axis=2)
    per = np.where(ok, np.concatenate([loc, (w / (1.0 + di))[:, :, None], ohk], axis=2), 0.0)
    cols.append(per.reshape(P, -1))
    return Qs, np.concatenate(cols, axis=1).astype(np.float32)


def atom_functions(basis):
    sh = basis.shells()
    natoms = len(basis.Z)
    types = [[] for _ in range(natoms)]
    first = [None] * natoms
    count = [0] * natoms
    for at, t, f0 in zip(sh["atom"], sh["type"], sh["first"]):
        types[at].append(int(t))
        if first[at] is None:
            first[at] = int(f0)
        count[at] += 1 if t == 0 else (3 if abs(t) == 1 else 2 * abs(t) + 1)
    return types, first, count


def pairs(xyz):
    xyz = np.asarray(xyz, dtype=np.float64)
    d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=2)
    a, b = np.nonzero(np.triu(d < CUTOFF))
    return [(int(i), int(j)) for i, j in zip(a, b)]


def supported(Z, basis):
    return all(z in ELEMENTS for z in Z) and basis.name == "def2-svp"


def sap_density(grid, H, S, nocc, metric=None, precision="fp64"):
    """Closed-shell density of the SAP guess (GuessSCF.cpp:17-75): occupied
    orbitals of H + V_SAP in the overlap metric.  The base the network
    corrects.  metric: overlap_metric(S) when the caller has it; precision
    "mixed" assembles V_SAP on the tensor cores."""
    from .scf import overlap_metric
    from ._lib import PRECISION_FP64, PRECISION_MIXED
    F = H + grid.sap_fock(PRECISION_MIXED if precision == "mixed" else PRECISION_FP64)
    X = (metric or overlap_metric(S))[0]
    _, C = np.linalg.eigh(X.T @ F @ X)
    Co = X @ C[:, :nocc]
    return 2.0 * Co @ Co.T


def dataset(Z, xyz, basis, D):
    """Features, local-frame targets and masks for every pair of a molecule
    with (converged - base) total density D."""
    types, first, count = atom_functions(basis)
    pr = pairs(xyz)
    Qs, Xf = frames_and_features(Z, xyz, pr)
    Ua, Ub = _pair_rotations(types, pr, Qs)
    X, T, Mk = [], [], []
    for p, ((a, b), Q) in enumerate(zip(pr, Qs)):
        blk = D[first[a]:first[a] + count[a], first[b]:first[b] + count[b]]
        loc = Ua[p] @ blk @ Ub[p].T
        t = np.zeros((MAX_FUNC, MAX_FUNC), dtype=np.float32)
        m = np.zeros_like(t)
        t[:count[a], :count[b]] = loc
        m[:count[a], :count[b]] = 1.0
        X.append(Xf[p])
        T.append(t.ravel())
        Mk.append(m.ravel())
    return np.array(X), np.array(T), np.array(Mk)


def _pair_rotations(types, pr, Qs):
    """Per pair (a, b): the atom rotations of a and b in the pair's frame.
    Each shell type's rotation is computed once for all frames, and each
    distinct atom layout's block-diagonal matrices once from those."""
    per_type = {t: shell_rotations(t, Qs) for t in sorted({t for ts in types for t in ts})}
    by_layout = {}
    for ts in {tuple(ts) for ts in types}:
        blocks = [per_type[t] for t in ts]
        n = sum(b.shape[1] for b in blocks)
        U = np.zeros((len(Qs), n, n))
        o = 0
        for b in blocks:
            k = b.shape[1]
            U[:, o:o + k, o:o + k] = b
            o += k
        by_layout[ts] = U
    keys_a = [tuple(types[a]) for a, _ in pr]
    keys_b = [tuple(types[b]) for _, b in pr]
    return _PairRotations(by_layout, keys_a), _PairRotations(by_layout, keys_b)


class _PairRotations(list):
    """Per-pair rotation matrices (a list, item p for pair p) that can also
    gather the pairs of one layout at once: take(idx) -> (len(idx), n, n)."""

    def __init__(self, by_layout, keys):
        super().__init__(by_layout[k][p] for p, k in enumerate(keys))
        self._by_layout, self._keys = by_layout, keys

    def take(self, idx):
        ks = {self._keys[p] for p in idx}
        if len(ks) != 1:
            return np.stack([self[p] for p in idx])
        return self._by_layout[ks.pop()][idx]


# ------------------------------------------------------------------ network

class PairMLP:
    """Device-resident MLP (include/chinium_guess.h)."""

    def __init__(self, nin=NIN, hidden=HIDDEN, layers=LAYERS, nout=NOUT, seed=0, params=None):
        self.nin, self.hidden, self.layers, self.nout = nin, hidden, layers, nout
        h = ctypes.c_void_p()
        check(lib().xc_mlp_create(nin, hidden, layers, nout, ctypes.byref(h)))
        self._h = h
        n = ctypes.c_long()
        check(lib().xc_mlp_nparams(h, ctypes.byref(n)))
        self.nparams = n.value
        self.set_params(params if params is not None else self.init_params(seed))
        self.residual = False  # True: targets are (converged - SAP) density blocks
        self.scale = 1.0       # network outputs are targets / scale

    def init_params(self, seed):
        rng = np.random.default_rng(seed)
        out = []
        dims = [self.nin] + [self.hidden] * self.layers + [self.nout]
        for fi, fo in zip(dims[:-1], dims[1:]):
            out.append((rng.normal(size=(fi, fo)) * math.sqrt(2.0 / fi)).ravel())
            out.append(np.zeros(fo))
        p = np.concatenate(out).astype(np.float32)
        assert len(p) == self.nparams
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().xc_mlp_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))

    def params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        check(lib().xc_mlp_get_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))
        return p

    def forward(self, X, bf16=False):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((len(X), self.nout), dtype=np.float32)
        check(lib().xc_mlp_forward(self._h, len(X), X.ctypes.data_as(ctypes.c_void_p),
                                   Y.ctypes.data_as(ctypes.c_void_p), int(bf16)))
        return Y

    def grad(self, X, dY):
        X = np.ascontiguousarray(X, dtype=np.float32)
        dY = np.ascontiguousarray(dY, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        check(lib().xc_mlp_backward(self._h, len(X), X.ctypes.data_as(ctypes.c_void_p),
                                    dY.ctypes.data_as(ctypes.c_void_p), g.ctypes.data_as(ctypes.c_void_p)))
        return g

    def train_step(self, X, T, M, lr):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        M = np.ascontiguousarray(M, dtype=np.float32)
        loss = ctypes.c_float()
        check(lib().xc_mlp_train_step(self._h, len(X), X.ctypes.data_as(ctypes.c_void_p),
                                      T.ctypes.data_as(ctypes.c_void_p), M.ctypes.data_as(ctypes.c_void_p),
                                      ctypes.c_float(lr), ctypes.byref(loss)))
        return loss.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xc_mlp_destroy(h)
            self._h = None


def train(model, X, T, M, epochs=200, batch=1024, lr=1e-3, seed=0, log=None):
    rng = np.random.default_rng(seed)
    n = len(X)
    losses = []
    for ep in range(epochs):
        perm = rng.permutation(n)
        tot = 0.0
        nb = 0
        lr_ep = lr * 0.5 * (1 + math.cos(math.pi * ep / epochs))
        for i in range(0, n, batch):
            idx = perm[i:i + batch]
            tot += model.train_step(X[idx], T[idx], M[idx], lr_ep)
            nb += 1
        losses.append(tot / max(nb, 1))
        if log and (ep % 20 == 0 or ep == epochs - 1):
            log("epoch %d loss %.3e" % (ep, losses[-1]))
    return losses


def assemble_blocks(pr, Y, Uas, Ubs, first, count, n):
    """The molecular-frame matrix from local pair blocks: block (a, b) =
    Ua^T y Ub and, for a != b, its transpose at (b, a); one batched product
    per (functions of a, functions of b) layout."""
    D = np.zeros((n, n))
    A = np.array([a for a, _ in pr])
    B = np.array([b for _, b in pr])
    ca_all = np.array([count[a] for a in A])
    cb_all = np.array([count[b] for b in B])
    fa, fb = np.array([first[a] for a in A]), np.array([first[b] for b in B])
    for ca, cb in sorted(set(zip(ca_all.tolist(), cb_all.tolist()))):
        idx = np.nonzero((ca_all == ca) & (cb_all == cb))[0]
        Ua = Uas.take(idx) if hasattr(Uas, "take") else np.stack([Uas[p] for p in idx])
        Ub = Ubs.take(idx) if hasattr(Ubs, "take") else np.stack([Ubs[p] for p in idx])
        blk = np.transpose(Ua, (0, 2, 1)) @ Y[idx, :ca, :cb].astype(np.float64) @ Ub
        rows = fa[idx][:, None] + np.arange(ca)
        cols = fb[idx][:, None] + np.arange(cb)
        D[rows[:, :, None], cols[:, None, :]] = blk
        off = A[idx] != B[idx]
        D[cols[off][:, :, None], rows[off][:, None, :]] = np.transpose(blk[off], (0, 2, 1))
    return D


def predict_density(model, Z, xyz, basis, S, nocc, bf16=True, D_base=None, metric=None, return_orbitals=False):
    """Learned closed-shell total density (2 C C^T, idempotent in the S metric):
    D_base (the SAP density for a residual model) plus the predicted pair
    blocks, purified.  metric: overlap_metric(S) when the caller has it.
    return_orbitals: also return the natural orbitals (S-orthonormal columns,
    occupied first), from which an SCF can rotate instead of diagonalising."""
    from .scf import overlap_metric
    types, first, count = atom_functions(basis)
    pr = pairs(xyz)
    Qs, X = frames_and_features(Z, xyz, pr)
    Y = model.forward(X, bf16=bf16).reshape(-1, MAX_FUNC, MAX_FUNC) * model.scale
    Uas, Ubs = _pair_rotations(types, pr, Qs)
    n = basis.nbasis
    if model.residual and D_base is None:
        raise ValueError("a residual model needs the base (SAP) density")
    D = assemble_blocks(pr, Y, Uas, Ubs, first, count, n)
    D = 0.5 * (D + D.T)
    if model.residual:
        D = D + D_base
    # purification: the projector onto the nocc most occupied natural orbitals
    # in the overlap metric -- by McWeeny iterations P <- 3P^2 - 2P^3 (GEMMs
    # only; the same projector when exactly nocc occupations exceed 1/2),
    # else (or when the orbitals are wanted) by diagonalisation
    _, Xh, Sh = metric or overlap_metric(S)
    P = 0.5 * (Sh @ D @ Sh)
    if not return_orbitals:
        converged = False
        for _ in range(12):
            P2 = P @ P
            if np.abs(P2 - P).max() < 1e-11:
                converged = True
                break
            P = 3.0 * P2 - 2.0 * (P2 @ P)
        if converged and abs(np.trace(P) - nocc) < 1e-7:
            P = 0.5 * (P + P.T)
            return 2.0 * (Xh @ P @ Xh)
        P = 0.5 * (Sh @ D @ Sh)
    occ, C = np.linalg.eigh(P)
    Cn = Xh @ C[:, np.argsort(occ)[::-1]]
    Co = Cn[:, :nocc]
    D = 2.0 * Co @ Co.T
    return (D, Cn) if return_orbitals else D


def guess_density(model, Z, xyz, ctx, bf16=True, precision="fp64", return_orbitals=False):
    """The learned starting density for a molecule whose SCF context (basis,
    S, H, grid) exists: the SAP base when the model is residual (its V_SAP on
    the tensor cores for precision "mixed").  return_orbitals: (D, natural
    orbitals), as predict_density."""
    from .scf import overlap_metric
    nocc = sum(Z) // 2
    metric = overlap_metric(ctx["S"], ctx)
    # tensor-core V_SAP only for a well-conditioned overlap (as the SCF's own SAP guess)
    prec = precision if ctx.get("S_min", 0.0) >= 1e-3 else "fp64"
    base = sap_density(ctx["grid"], ctx["H"], ctx["S"], nocc, metric, prec) if model.residual else None
    return predict_density(model, Z, xyz, ctx["basis"], ctx["S"], nocc, bf16=bf16, D_base=base, metric=metric,
                           return_orbitals=return_orbitals)


def save(model, path):
    np.savez_compressed(path, params=model.params(), shape=np.array([model.nin, model.hidden, model.layers, model.nout]),
                        residual=np.array(int(model.residual)), scale=np.array(model.scale))


def load(path):
    d = np.load(path)
    nin, hidden, layers, nout = (int(v) for v in d["shape"])
    m = PairMLP(nin, hidden, layers, nout, params=d["params"])
    m.residual = bool(int(d["residual"])) if "residual" in d else False
    m.scale = float(d["scale"]) if "scale" in d else 1.0
    return m


DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "guess_water_def2svp.npz")
_DEFAULT = None


def default_model():
    """The packaged network (loaded once per process)."""
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = load(DEFAULT_WEIGHTS)
    return _DEFAULT
