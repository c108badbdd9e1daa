"""SCF checkpoints: the converged density matrices as raw FP64 next to JSON
metadata, for a restart or a later guess.

The reference exports its wavefunction to <job>.mwfn after an SCF
(SelfConsistentField.h:25-30) and reads it back with `guess READ`
(Representation.cpp:24-29); libmwfn is absent here, so the checkpoint is the
density itself: <path>.bin holds the nspin n x n matrices (row-major, total
density for restricted runs, [D_alpha, D_beta] otherwise) and <path>.json the
molecule, basis, functional, grid, charge, multiplicity, energy and a SHA-256
of the payload.  load_checkpoint checks what the caller states against the
metadata and returns what run_scf takes as `guess`.
"""
import hashlib
import json
import os

import numpy as np

FORMAT = "chinium_gb300 density checkpoint"
VERSION = 1


def save_checkpoint(path, result, Z, xyz_bohr, basis, functional, grid, charge=0, mult=1):
    """Write result.D (a run_scf result) to <path>.bin and <path>.json."""
    D = np.ascontiguousarray(np.stack([np.asarray(d, dtype=np.float64) for d in result.D]))
    payload = D.tobytes()
    meta = {
        "format": FORMAT, "version": VERSION, "dtype": "float64", "layout": "row-major (nspin, n, n)",
        "Z": [int(z) for z in Z], "xyz_bohr": np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3).tolist(),
        "basis": basis, "functional": functional, "grid": grid, "charge": int(charge), "mult": int(mult),
        "nspin": int(D.shape[0]), "nbasis": int(D.shape[1]),
        "energy": float(result.energy), "converged": bool(result.converged), "iterations": int(result.iterations),
        "sha256": hashlib.sha256(payload).hexdigest(),
    }
    tmp_bin, tmp_json = path + ".bin.tmp", path + ".json.tmp"
    with open(tmp_bin, "wb") as f:
        f.write(payload)
    with open(tmp_json, "w") as f:
        json.dump(meta, f, indent=1)
    os.replace(tmp_bin, path + ".bin")  # the payload first: a complete .json always has its .bin
    os.replace(tmp_json, path + ".json")
    return meta


def load_checkpoint(path, Z=None, basis=None, nbasis=None, charge=None, mult=None, xyz_bohr=None,
                    geometry_tol=None):
    """The densities of a checkpoint as a run_scf guess (the total density for
    one spin, [D_alpha, D_beta] for two) and its metadata.  Every argument given
    must match the metadata (ValueError otherwise); xyz_bohr is compared only
    when geometry_tol is set (a density from a nearby geometry is still a
    good guess)."""
    with open(path + ".json") as f:
        meta = json.load(f)
    if meta.get("format") != FORMAT or meta.get("version") != VERSION:
        raise ValueError("not a %s (version %d): %s" % (FORMAT, VERSION, path))
    with open(path + ".bin", "rb") as f:
        payload = f.read()
    if hashlib.sha256(payload).hexdigest() != meta["sha256"]:
        raise ValueError("checkpoint payload does not match its checksum: %s.bin" % path)
    ns, n = meta["nspin"], meta["nbasis"]
    if len(payload) != 8 * ns * n * n:
        raise ValueError("checkpoint payload has the wrong size")
    for key, want in (("Z", None if Z is None else [int(z) for z in Z]), ("basis", basis), ("nbasis", nbasis),
                      ("charge", charge), ("mult", mult)):
        if want is not None and meta[key] != want:
            raise ValueError("checkpoint %s is %r, not %r" % (key, meta[key], want))
    if geometry_tol is not None and xyz_bohr is not None:
        d = np.abs(np.asarray(meta["xyz_bohr"]) - np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)).max()
        if d > geometry_tol:
            raise ValueError("checkpoint geometry differs by %.3g bohr" % d)
    D = np.frombuffer(payload, dtype=np.float64).reshape(ns, n, n).copy()
    return (D[0] if ns == 1 else [D[0], D[1]]), meta
