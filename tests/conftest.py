import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the product kernels)")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def h2o_oracle():
    """H2O / def2-SVP / SG-1 through the oracle (grid, blocks, AO)."""
    from oracle import oracle as O
    from chinium_gb300 import molecules as M
    Z, xyz = M.h2o()
    basis = O.Basis(Z, xyz, "def2-svp")
    grid = O.OracleGrid(basis, "SG-1", Z, xyz)
    return Z, xyz, basis, grid


def grid_overlap(grid):
    n = grid.basis.nbasis
    S = np.zeros((n, n))
    for (bx, by, bz, bw), (ao, _) in zip(grid.blocks, grid.ao):
        S += (ao * bw) @ ao.T
    return S


def model_density(grid, nocc, seed=0, nspin=1):
    """Physically shaped density matrices: occupied orbitals of a random
    symmetric one-electron operator, orthonormal in the grid overlap metric.
    Returns the total density 2 C C^T (nspin=1) or [Da, Db]."""
    import scipy.linalg
    rng = np.random.default_rng(seed)
    S = grid_overlap(grid)
    n = S.shape[0]
    H = rng.normal(size=(n, n))
    H = H + H.T + np.diag(np.linspace(-5, 5, n))
    _, C = scipy.linalg.eigh(H, S)
    if nspin == 1:
        Co = C[:, :nocc]
        return 2 * Co @ Co.T
    na, nb = nocc
    return [C[:, :na] @ C[:, :na].T, C[:, :nb] @ C[:, :nb].T]
