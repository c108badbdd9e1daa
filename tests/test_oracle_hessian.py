"""The oracle's Hessian skeleton terms on the CPU.  getFockSkeleton
(GridFock.cpp:52-95) plus getFockU<s_t> on the skeleton density derivatives of
getDensitySkeleton (GridDensity.cpp:79-130) is dV_xc / dR_(A,t) at fixed D with
the grid held fixed, which central differences of the oracle's V_xc with one
atom's basis functions displaced give independently (Richardson, steps 1e-4
and 5e-5 bohr); getDensitySkeleton2 + getEnergyHess (restricted) is
d^2 E_xc / dR dR at fixed D, checked against second differences of E_xc.  The
energy Hessian has no device counterpart yet: it is the parity target for one."""
import numpy as np
import pytest

from conftest import model_density
from oracle import oracle as O


@pytest.mark.parametrize("name,nspin", [("SVWN5", 1), ("PBE", 1), ("PBE", 2), ("BLYP", 2)])
def test_skeleton_fock_terms_are_the_fixed_density_derivative_of_fock(h2o_oracle, name, nspin):
    Z, xyz, basis, og = h2o_oracle
    ids = O.FUNCTIONAL_FILES[name]
    D = model_density(og, 5)[None] if nspin == 1 else np.stack(model_density(og, (5, 4), nspin=2, seed=2))
    Fs, Fu = og.fock_skeleton(D, ids, nspin)
    ref = O.fock_fd(og, Z, xyz, "def2-svp", D, ids, nspin)
    err = np.abs(Fs + Fu - ref).max()
    assert err < 2e-10, (name, nspin, err)
    # both parts matter, and both are symmetric
    assert np.abs(Fs).max() > 0.1 and np.abs(Fu).max() > 0.1
    assert np.abs(Fs - Fs.transpose(0, 1, 3, 2)).max() < 1e-14
    assert np.abs(Fu - Fu.transpose(0, 1, 3, 2)).max() < 1e-13


def test_ao_second_derivatives_match_differences_of_gradients(h2o_oracle):
    Z, xyz, basis, og = h2o_oracle
    bx, by, bz, _ = og.blocks[3]
    a2 = basis.ao2(bx, by, bz)
    fd = np.zeros_like(a2)
    for b, dv in enumerate(np.eye(3) * 1e-5):
        d = (basis.ao(bx + dv[0], by + dv[1], bz + dv[2], 1)[1] - basis.ao(bx - dv[0], by - dv[1], bz - dv[2], 1)[1]) / 2e-5
        for a in range(b + 1):
            fd[a + b * (b + 1) // 2] = d[a]
    scale = np.abs(a2).max()
    assert scale > 1.0
    assert np.abs(a2 - fd).max() < 1e-6 * scale
    # the Laplacian of the functions is the trace xx + yy + zz
    assert np.all(np.isfinite(a2[0] + a2[2] + a2[5]))


@pytest.mark.parametrize("name", ["SVWN5", "PBE"])
def test_energy_hessian_matches_second_differences(h2o_oracle, name):
    """getDensitySkeleton2 + getEnergyHess restated (restricted): d^2 E_xc / dR_i dR_j at fixed D
    with the grid fixed, against four-point differences of the oracle's E_xc with the basis
    functions displaced (steps 2.5e-4 and 1.25e-4 bohr, Richardson: the oxygen core needs the
    small steps) on same-atom, cross-atom and same-coordinate pairs."""
    Z, xyz, basis, og = h2o_oracle
    ids = O.FUNCTIONAL_FILES[name]
    D = model_density(og, 5)
    H = O.energy_hess(og, D, ids)
    assert np.abs(H - H.T).max() < 1e-12
    pairs = [(0, 0), (0, 1), (2, 2), (0, 3), (3, 4), (5, 8), (4, 7), (8, 8)]
    ref = O.energy_hess_fd(og, Z, xyz, "def2-svp", D, ids, pairs, h=2.5e-4)
    for (i, j), v in ref.items():
        assert abs(H[i, j] - v) < 2e-6, (name, i, j, H[i, j], v)
    assert np.all(np.isfinite(H))


def test_ao_third_derivatives_match_differences_of_second(h2o_oracle):
    Z, xyz, basis, og = h2o_oracle
    bx, by, bz, _ = og.blocks[3]
    a3 = basis.ao3(bx, by, bz)

    def tp(a, b, c):
        v = sorted((a, b, c))
        return v[0] + v[1] * (v[1] + 1) // 2 + v[2] * (v[2] + 1) * (v[2] + 2) // 6

    fd = np.zeros_like(a3)
    for c, dv in enumerate(np.eye(3) * 1e-5):
        d = (basis.ao2(bx + dv[0], by + dv[1], bz + dv[2]) - basis.ao2(bx - dv[0], by - dv[1], bz - dv[2])) / 2e-5
        for b in range(3):
            for a in range(b + 1):
                fd[tp(a, b, c)] = d[a + b * (b + 1) // 2]
    assert np.abs(a3 - fd).max() < 1e-7 * np.abs(a3).max()
