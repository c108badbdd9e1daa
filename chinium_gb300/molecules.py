"""Synthetic molecules with the shapes of the benchmark configurations.

All coordinates are returned in bohr (the reference converts its angstrom
input with 1.8897259886, src/Macro/Unit.h:1).  Every generator is seeded and
deterministic.
"""
import math

import numpy as np

ANGSTROM2BOHR = 1.8897259886
TETRA = math.degrees(math.acos(-1.0 / 3.0))  # 109.4712...


def h2o():
    """O (0, 0, 0.1173), H (0, +-0.7572, -0.4692) angstrom."""
    xyz = np.array([[0.0, 0.0, 0.1173], [0.0, 0.7572, -0.4692], [0.0, -0.7572, -0.4692]])
    return [8, 1, 1], xyz * ANGSTROM2BOHR


def c18(radius=3.88, bonds=(1.22, 1.35)):
    """cyclo[18]carbon on a ring of the given radius.  The two arc angles
    alternate and close the ring (9 (a + b) = 2 pi) with chord lengths in the
    ratio of the two bond lengths; a ring of radius 3.88 A cannot hold chords
    of exactly 1.22 and 1.35 A, so the ratio is kept and the radius wins."""
    r1, r2 = bonds
    lo, hi = 0.0, 2 * math.pi / 9
    for _ in range(200):  # solve sin(a/2) / sin(b/2) = r1 / r2 with b = 2 pi / 9 - a
        a = 0.5 * (lo + hi)
        b = 2 * math.pi / 9 - a
        if math.sin(a / 2) / math.sin(b / 2) < r1 / r2:
            lo = a
        else:
            hi = a
    a = 0.5 * (lo + hi)
    b = 2 * math.pi / 9 - a
    ang, xyz = 0.0, []
    for i in range(18):
        xyz.append([radius * math.cos(ang), radius * math.sin(ang), 0.0])
        ang += a if i % 2 == 0 else b
    return [6] * 18, np.array(xyz) * ANGSTROM2BOHR


def _place(a, b, c, bond, angle_deg, torsion_deg):
    """Natural extension reference frame: position of d bonded to c with
    |cd| = bond, angle bcd and torsion abcd."""
    ang = math.radians(angle_deg)
    tor = math.radians(torsion_deg)
    bc = c - b
    bc /= np.linalg.norm(bc)
    n = np.cross(b - a, bc)
    n /= np.linalg.norm(n)
    m = np.cross(n, bc)
    d2 = np.array([-bond * math.cos(ang), bond * math.sin(ang) * math.cos(tor), bond * math.sin(ang) * math.sin(tor)])
    return c + d2[0] * bc + d2[1] * m + d2[2] * n


def _hydrogens(center, neighbours, nh, ch):
    """Directions completing a tetrahedron around a carbon."""
    us = [(nb - center) / np.linalg.norm(nb - center) for nb in neighbours]
    out = []
    if len(us) == 0:
        for v in ([1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]):
            out.append(center + ch * np.array(v) / math.sqrt(3))
        return out[:nh]
    if len(us) == 1:
        ax = -us[0]
        p = np.cross(ax, [0.0, 0.0, 1.0])
        if np.linalg.norm(p) < 1e-6:
            p = np.cross(ax, [0.0, 1.0, 0.0])
        p /= np.linalg.norm(p)
        q = np.cross(ax, p)
        th = math.radians(180.0 - TETRA)
        for k in range(3):
            ph = 2 * math.pi * k / 3
            d = ax * math.cos(th) + (p * math.cos(ph) + q * math.sin(ph)) * math.sin(th)
            out.append(center + ch * d)
        return out[:nh]
    bis = -(us[0] + us[1])
    bis /= np.linalg.norm(bis)
    nrm = np.cross(us[0], us[1])
    nrm /= np.linalg.norm(nrm)
    al = math.radians(TETRA / 2)
    for sgn in (1, -1):
        out.append(center + ch * (bis * math.cos(al) + sgn * nrm * math.sin(al)))
    return out[:nh]


def alkane(n, rng, cc=1.53, ch=1.09, min_sep=1.6):
    """Linear C_nH_(2n+2), tetrahedral angles, torsions uniform in [0, 360).
    A torsion is redrawn (up to 200 times, keeping the best draw) while it
    brings two non-bonded atoms closer than min_sep angstrom; the draw
    sequence, and so the molecule, is fixed by rng."""
    carbons = [np.zeros(3)]
    if n >= 2:
        carbons.append(np.array([cc, 0.0, 0.0]))
    if n >= 3:
        th = math.radians(180 - TETRA)
        carbons.append(carbons[1] + cc * np.array([math.cos(th), math.sin(th), 0.0]))

    def hydrogens_of(i, cs):
        nbrs = [cs[j] for j in (i - 1, i + 1) if 0 <= j < len(cs)]
        return _hydrogens(cs[i], nbrs, 4 - len(nbrs), ch)

    # atoms whose positions are final: carbons placed so far and the
    # hydrogens of every carbon whose two neighbours are known
    fixed = [c for c in carbons]
    fixed_owner = [i for i in range(len(carbons))]
    nfinal_h = max(0, len(carbons) - 1) if n > len(carbons) else 0
    for i in range(nfinal_h):
        for h in hydrogens_of(i, carbons):
            fixed.append(h)
            fixed_owner.append(i)

    def min_sep_of(new_atoms, new_owner):
        F = np.array(fixed)
        fo = np.array(fixed_owner)
        best = np.inf
        for a, oa, is_c in new_atoms:
            d = np.linalg.norm(F - a, axis=1)
            # skip bonded pairs: C-C neighbours, a hydrogen and its carbon
            skip = (fo == oa) | ((np.arange(len(F)) < len(carbons)) & is_c & (np.abs(fo - oa) == 1))
            if is_c:
                skip |= (fo == oa - 1) & (np.arange(len(F)) < len(carbons))
            d = np.where(skip, np.inf, d)
            best = min(best, d.min() if len(d) else np.inf)
        return best

    for i in range(3, n):
        best, best_sep = None, -1.0
        for _ in range(200):
            cand = _place(carbons[i - 3], carbons[i - 2], carbons[i - 1], cc, TETRA, rng.uniform(0, 360))
            trial = carbons + [cand]
            new = [(cand, i, True)] + [(h, i - 1, False) for h in hydrogens_of(i - 1, trial)]
            if i == n - 1:  # the last carbon's hydrogens are final too
                new += [(h, i, False) for h in hydrogens_of(i, trial)]
            sep = min_sep_of(new, None)
            if sep > best_sep:
                best, best_sep = cand, sep
            if sep >= min_sep:
                break
        carbons.append(best)
        fixed.append(best)
        fixed_owner.append(i)
        for h in hydrogens_of(i - 1, carbons):
            fixed.append(h)
            fixed_owner.append(i - 1)
    Z, xyz = [], []
    for c in carbons:
        Z.append(6)
        xyz.append(c)
    for i in range(n):
        for h in hydrogens_of(i, carbons):
            Z.append(1)
            xyz.append(h)
    return Z, np.array(xyz) * ANGSTROM2BOHR


_BATCH_CACHE = {}


def alkane_batch(count=64, seed=0, nmin=1, nmax=20):
    """count linear alkanes with n ~ U{nmin..nmax} and random torsions (seed)."""
    key = (count, seed, nmin, nmax)
    if key not in _BATCH_CACHE:
        rng = np.random.default_rng(seed)
        ns = rng.integers(nmin, nmax + 1, size=count)
        _BATCH_CACHE[key] = [alkane(int(k), rng) for k in ns]
    return [(list(Z), xyz.copy()) for Z, xyz in _BATCH_CACHE[key]]


def fe4s4(fe_s=2.28, fe_fe=2.75):
    """Fe4S4 cubane: Fe on tetrahedron vertices, S on the inverted
    tetrahedron, Fe-S fixed; the Fe-Fe distance fixes the remaining freedom."""
    a = fe_fe / (2 * math.sqrt(2))
    # (a + b)^2 + 2 (a - b)^2 = fe_s^2
    b = (2 * a + math.sqrt(4 * a * a - 12 * (3 * a * a - fe_s * fe_s))) / 6
    tet = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=float)
    xyz = np.vstack([a * tet, -b * tet])
    return [26] * 4 + [16] * 4, xyz * ANGSTROM2BOHR


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_cluster(k, rng, oo_min=2.6, oo_max=3.2):
    """(H2O)_k: rigid monomers (geometry of h2o()), random orientations, each
    new oxygen 2.6-3.2 A from a random earlier oxygen and >= 2.6 A from all."""
    _, mono = h2o()
    mono = mono / ANGSTROM2BOHR
    mono = mono - mono[0]
    Z, xyz = [], []
    oxygens = []
    for m in range(k):
        for _ in range(1000):
            R = _rotation(rng)
            if not oxygens:
                o = np.zeros(3)
            else:
                anchor = oxygens[rng.integers(len(oxygens))]
                d = rng.normal(size=3)
                d /= np.linalg.norm(d)
                o = anchor + d * rng.uniform(oo_min, oo_max)
            atoms = mono @ R.T + o
            if oxygens and min(np.linalg.norm(o - p) for p in oxygens) < oo_min:
                continue
            if xyz and min(np.linalg.norm(a - b) for a in atoms for b in xyz) < 1.4:
                continue
            break
        oxygens.append(o)
        Z += [8, 1, 1]
        xyz += list(atoms)
    return Z, np.array(xyz) * ANGSTROM2BOHR


def water_clusters(count, seed, kmin=2, kmax=8):
    rng = np.random.default_rng(seed)
    ks = rng.integers(kmin, kmax + 1, size=count)
    return [water_cluster(int(k), rng) for k in ks]


def nuclear_repulsion(Z, xyz):
    Z = np.asarray(Z, dtype=float)
    e = 0.0
    for i in range(len(Z)):
        for j in range(i):
            e += Z[i] * Z[j] / np.linalg.norm(xyz[i] - xyz[j])
    return e
