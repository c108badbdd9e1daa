"""Regenerates the package's data tables from a Chinium source tree.

Run once in a container that has the reference tree (path given by
``--ref``, default ``$CHINIUM_PATH``); the outputs are committed so that the
library and tests need no reference tree at run time.

Outputs (all plain text, written next to this script):

* ``lebedev.txt`` -- Lebedev-Laikov angular rules for every order any SG-n
  recipe uses.  The tables come from running the reference's own
  ``src/Grid/sphere_lebedev_rule.cpp`` (compiled in place by
  ``oracle/Makefile`` target ``ref``), called exactly like
  ``src/Grid/GridGeneration.cpp:121-125`` calls ``ld_by_order``.
* ``grids/SG-{1,2,3}.txt`` -- per-element radial/angular recipes, the fields of
  ``Grids/SG-n/<El>.grid`` (format documented in ``Grids/README.md``).
* ``basis/<name>.txt`` -- contracted Gaussian shells per element, parsed from
  ``BasisSets/<name>.gbs`` (Gaussian format; ``D`` exponents; ``SP`` shells
  split into an S and a P shell sharing exponents).
* ``functionals.txt`` -- the libxc ids listed by each
  ``DensityFunctionals/<NAME>.df`` (read at src/ExchangeCorrelation.cpp:18-34).
* ``sap.txt`` -- the tabulated SAP radial potentials
  (``src/HartreeFockKohnSham/SAP/v_*.dat`` and ``v_Radii.dat``, indexed as in
  ``src/HartreeFockKohnSham/SAP.h``).
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

SYMBOLS = [
    "X", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S",
    "Cl", "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge",
    "As", "Se", "Br", "Kr",
]
BASIS_SETS = ["def2-svp", "def2-tzvp", "sto-3g", "6-31g"]
MAX_Z = 36


def read_grid_recipes(ref, name):
    out = []
    folder = os.path.join(ref, "Grids", name)
    for z in range(1, MAX_Z + 1):
        path = os.path.join(folder, SYMBOLS[z] + ".grid")
        if not os.path.exists(path):
            continue
        with open(path) as f:
            lines = [ln.split("#")[0].strip() for ln in f]
        lines = [ln for ln in lines if ln]
        ngroups, nshells = (int(t) for t in lines[0].split()[:2])
        radial = lines[1].split()
        groups = [tuple(int(t) for t in ln.split()[:2]) for ln in lines[2:2 + ngroups]]
        # SG-2/Si.grid declares 75 shells but its groups hold 78; the reference
        # uses the declared total for the radial step and walks all groups.
        out.append((z, nshells, radial, groups))
    return out


def read_gbs(path):
    shells_by_z = {}
    with open(path) as f:
        lines = [ln.rstrip() for ln in f]
    i = 0
    cur = None
    while i < len(lines):
        ln = lines[i].strip()
        i += 1
        if not ln or ln.startswith("!"):
            continue
        if ln.startswith("****"):
            cur = None
            continue
        toks = ln.split()
        if cur is None:
            # element header '-Sym 0' (or 'Sym 0'); elements beyond the table
            # are skipped up to their '****' terminator
            sym = toks[0].lstrip("-")
            sym = sym[0].upper() + sym[1:].lower()
            cur = SYMBOLS.index(sym) if sym in SYMBOLS else -1
            if cur > 0:
                shells_by_z[cur] = []
            continue
        if cur < 0:
            continue
        kind = toks[0].upper()
        nprim = int(toks[1])
        rows = []
        for _ in range(nprim):
            vals = [float(t.replace("D", "E").replace("d", "e")) for t in lines[i].split()]
            rows.append(vals)
            i += 1
        if kind == "SP":
            shells_by_z[cur].append(("S", [r[0] for r in rows], [r[1] for r in rows]))
            shells_by_z[cur].append(("P", [r[0] for r in rows], [r[2] for r in rows]))
        else:
            shells_by_z[cur].append((kind, [r[0] for r in rows], [r[1] for r in rows]))
    return shells_by_z


def read_sap(ref):
    folder = os.path.join(ref, "src", "HartreeFockKohnSham", "SAP")

    def load(fn):
        with open(os.path.join(folder, fn)) as f:
            txt = f.read()
        vals = [float(t) for t in re.split(r"[,\s]+", txt) if t]
        assert len(vals) == 751, fn
        return vals

    radii = load("v_Radii.dat")
    pots = {z: load("v_%s.dat" % SYMBOLS[z]) for z in range(1, MAX_Z + 1)}
    return radii, pots


def lebedev_tables(ref, orders):
    exe = os.path.join(REPO, "oracle", "_ref", "lebedev_dump")
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + ref])
    return subprocess.check_output([exe] + [str(o) for o in orders]).decode()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CHINIUM_PATH", ""))
    args = ap.parse_args()
    ref = args.ref
    if not ref or not os.path.isdir(ref):
        sys.exit("reference tree not found; pass --ref")

    os.makedirs(os.path.join(HERE, "grids"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "basis"), exist_ok=True)

    orders = set()
    for name in ("SG-1", "SG-2", "SG-3"):
        recipes = read_grid_recipes(ref, name)
        with open(os.path.join(HERE, "grids", name + ".txt"), "w") as f:
            f.write("# per element: Z nshells_total radial-formula params... ; then ngroups lines 'npoints nshells'\n")
            for z, nshells, radial, groups in recipes:
                f.write("element %d %d %d %s\n" % (z, nshells, len(groups), " ".join(radial)))
                for npts, nsh in groups:
                    f.write("%d %d\n" % (npts, nsh))
                    orders.add(npts)

    with open(os.path.join(HERE, "lebedev.txt"), "w") as f:
        f.write(lebedev_tables(ref, sorted(orders)))

    for bs in BASIS_SETS:
        shells = read_gbs(os.path.join(ref, "BasisSets", bs + ".gbs"))
        with open(os.path.join(HERE, "basis", bs + ".txt"), "w") as f:
            f.write("# contracted Gaussian shells per element: 'element Z nshells', then 'L nprim' + nprim 'exponent coefficient'\n")
            for z in sorted(shells):
                if z > MAX_Z:
                    continue
                f.write("element %d %d\n" % (z, len(shells[z])))
                for kind, exps, coefs in shells[z]:
                    lval = "SPDFGHI".index(kind)
                    f.write("%d %d\n" % (lval, len(exps)))
                    for e, c in zip(exps, coefs):
                        f.write("%.17g %.17g\n" % (e, c))

    with open(os.path.join(HERE, "functionals.txt"), "w") as f:
        f.write("# DensityFunctionals/<NAME>.df: NAME followed by its libxc ids\n")
        folder = os.path.join(ref, "DensityFunctionals")
        for fn in sorted(os.listdir(folder)):
            if fn.endswith(".df"):
                with open(os.path.join(folder, fn)) as g:
                    ids = g.readline().split()
                f.write(fn[:-3] + " " + " ".join(ids) + "\n")

    radii, pots = read_sap(ref)
    with open(os.path.join(HERE, "sap.txt"), "w") as f:
        f.write("# SAP radial table: first line 'radii' + 751 values, then 'Z' + 751 values of r*V(r)\n")
        f.write("radii " + " ".join("%.10e" % v for v in radii) + "\n")
        for z in sorted(pots):
            f.write("%d " % z + " ".join("%.10e" % v for v in pots[z]) + "\n")


if __name__ == "__main__":
    main()
