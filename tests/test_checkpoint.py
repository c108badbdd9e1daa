"""SCF checkpoints on the CPU: round trip, metadata checks, corruption."""
import numpy as np
import pytest

from chinium_gb300.checkpoint import load_checkpoint, save_checkpoint
from chinium_gb300.scf import Result


def fake_result(nspin, n, seed=0):
    rng = np.random.default_rng(seed)
    Ds = []
    for _ in range(nspin):
        A = rng.normal(size=(n, n))
        Ds.append(A + A.T)
    return Result(D=Ds, energy=-76.123456789, converged=True, iterations=11)


@pytest.mark.parametrize("nspin", [1, 2])
def test_checkpoint_round_trip(tmp_path, nspin):
    r = fake_result(nspin, 24)
    Z, xyz = [8, 1, 1], np.array([[0, 0, 0.22], [0, 1.43, -0.89], [0, -1.43, -0.89]])
    p = str(tmp_path / "h2o")
    save_checkpoint(p, r, Z, xyz, "def2-svp", "PBE", "SG-1", mult=1 if nspin == 1 else 3)
    D, meta = load_checkpoint(p, Z=Z, basis="def2-svp", nbasis=24, xyz_bohr=xyz, geometry_tol=1e-12)
    got = [D] if nspin == 1 else D
    for a, b in zip(got, r.D):
        assert np.array_equal(a, b)
    assert meta["energy"] == r.energy and meta["nspin"] == nspin and meta["functional"] == "PBE"


def test_checkpoint_rejects_mismatch_and_corruption(tmp_path):
    r = fake_result(1, 24)
    Z, xyz = [8, 1, 1], np.zeros((3, 3))
    p = str(tmp_path / "c")
    save_checkpoint(p, r, Z, xyz, "def2-svp", "PBE", "SG-1")
    with pytest.raises(ValueError):
        load_checkpoint(p, basis="def2-tzvp")
    with pytest.raises(ValueError):
        load_checkpoint(p, Z=[8, 1])
    with pytest.raises(ValueError):
        load_checkpoint(p, xyz_bohr=xyz + 0.1, geometry_tol=1e-3)
    load_checkpoint(p, xyz_bohr=xyz + 0.1)  # no tolerance given: a nearby geometry's density is a guess
    with open(p + ".bin", "r+b") as f:
        f.seek(100)
        f.write(b"\x00\x01")
    with pytest.raises(ValueError):
        load_checkpoint(p)
