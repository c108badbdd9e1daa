"""Generates tests/golden/reference_facts.json from a Chinium source tree.

Every number comes from the reference's own files or code, not from this
project's restatement:
  * grid point counts per configuration by the reference's counting rule
    (SphericalGridNumber, src/Grid/GridGeneration.cpp:27-48: sum over atoms and
    groups of nshells * npoints read from Grids/SG-n/<El>.grid);
  * the block partition sizes that RecursiveCut (GridGeneration.cpp:203-210,
    halving at max_size = 128, :24) and the pad to a multiple of 8 (:212-214)
    produce for those counts;
  * basis sizes from BasisSets/*.gbs with pure d/f and Cartesian p;
  * Lebedev checksums by running the reference's sphere_lebedev_rule.cpp
    (compiled in place by oracle/Makefile target `ref`).

Usage: python tests/golden/make_golden.py --ref /path/to/chinium
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from chinium_gb300 import molecules as M  # noqa: E402

SYM = ["X", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S",
       "Cl", "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe"]


def grid_count(ref, grid, Z):
    n = 0
    for z in Z:
        with open(os.path.join(ref, "Grids", grid, SYM[z] + ".grid")) as f:
            lines = [ln.split("#")[0].split() for ln in f]
        lines = [ln for ln in lines if ln]
        ng = int(lines[0][0])
        for ln in lines[2:2 + ng]:
            n += int(ln[0]) * int(ln[1])
    return n


def blocks(n):
    out = []

    def rec(k):
        if k <= 128:
            out.append(k)
        else:
            rec(k // 2)
            rec(k - k // 2)

    rec(n)
    return out


def nbasis(ref, basis, Z):
    size = {"S": 1, "P": 3, "D": 5, "F": 7, "G": 9, "SP": 4}
    per = {}
    with open(os.path.join(ref, "BasisSets", basis + ".gbs")) as f:
        lines = [ln.strip() for ln in f]
    cur = None
    i = 0
    while i < len(lines):
        ln = lines[i]
        i += 1
        if not ln or ln.startswith("!"):
            continue
        if ln.startswith("****"):
            cur = None
            continue
        t = ln.split()
        if cur is None:
            s = t[0].lstrip("-")
            cur = s[0].upper() + s[1:].lower()
            per[cur] = 0
            continue
        per[cur] += size[t[0].upper()]
        i += int(t[1])
    return sum(per[SYM[z]] for z in Z)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CHINIUM_PATH", ""))
    ref = ap.parse_args().ref
    facts = {"configs": {}}
    cases = {
        "h2o_svp_sg1": (M.h2o(), "def2-svp", "SG-1"),
        "c18_tzvp_sg2": (M.c18(), "def2-tzvp", "SG-2"),
        "fe4s4_tzvp_sg3": (M.fe4s4(), "def2-tzvp", "SG-3"),
        "ch4_svp_sg2": (M.alkane(1, None), "def2-svp", "SG-2"),
    }
    for name, ((Z, _), bs, grid) in cases.items():
        G = grid_count(ref, grid, Z)
        b = blocks(G)
        facts["configs"][name] = {
            "Z": Z, "basis": bs, "grid": grid, "npoints": G, "nblocks": len(b),
            "npoints_padded": sum((k + 7) & ~7 for k in b), "min_block": min(b), "max_block": max(b),
            "nbasis": nbasis(ref, bs, Z),
        }
    exe = os.path.join(REPO, "oracle", "_ref", "lebedev_dump")
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + ref])
    orders = [6, 26, 38, 50, 86, 110, 146, 194, 302, 590]
    out = subprocess.check_output([exe] + [str(o) for o in orders]).decode().split("\n")
    sums = {}
    i = 0
    while i < len(out):
        if out[i].startswith("order"):
            n = int(out[i].split()[1])
            rows = [[float(v) for v in out[i + 1 + k].split()] for k in range(n)]
            sums[n] = {"sum_w": sum(r[3] for r in rows), "sum_wz2": sum(r[3] * r[2] ** 2 for r in rows),
                       "sum_abs_x": sum(abs(r[0]) for r in rows)}
            i += n + 1
        else:
            i += 1
    facts["lebedev"] = sums
    with open(os.path.join(HERE, "reference_facts.json"), "w") as f:
        json.dump(facts, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
