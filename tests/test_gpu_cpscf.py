"""Coupled-perturbed Kohn-Sham end to end: the static polarizability of H2O
from CPKS with the XC response of Evaluate("f") + getDensityU + getFockU<u_t>
against finite-field SCF energies (-d^2 E / d F^2, Richardson-extrapolated
central differences), and the tensor-core response against the FP64 one."""
import numpy as np
import pytest

from chinium_gb300 import molecules as M
from chinium_gb300.cpscf import finite_field_polarizability, polarizability
from chinium_gb300.scf import run_scf

pytestmark = pytest.mark.gpu

KW = dict(grid="SG-1", jk_device="cpu")


@pytest.fixture(scope="module", params=["PBE", "B3LYP"])
def water(request):
    Z, xyz = M.h2o()
    scf = run_scf(Z, xyz, functional=request.param, conv_energy=1e-12, conv_grad=1e-9, **KW)
    assert scf.converged
    return request.param, Z, xyz, scf


def test_cpks_polarizability_matches_finite_field(water):
    name, Z, xyz, scf = water
    alpha, iters = polarizability(Z, xyz, scf, name)
    print(name, "alpha diag", np.diag(alpha), "iterations", iters)
    assert np.abs(alpha - alpha.T).max() < 1e-7
    assert np.all(np.diag(alpha) > 1.0)
    for axis in range(3):
        ff = finite_field_polarizability(Z, xyz, scf, name, axis, **KW)
        print(name, axis, "CPKS %.8f  finite field %.8f" % (alpha[axis, axis], ff))
        assert abs(alpha[axis, axis] - ff) < 2e-5


def test_cpks_mixed_response_matches_fp64(water):
    name, Z, xyz, scf = water
    a64, _ = polarizability(Z, xyz, scf, name)
    amx, _ = polarizability(Z, xyz, scf, name, precision="mixed")
    print(name, "max |d alpha| mixed vs fp64 %.2e" % np.abs(amx - a64).max())
    assert np.abs(amx - a64).max() < 1e-5 * np.abs(a64).max()
