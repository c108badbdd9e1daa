"""Learned starting density: host logic on CPU (frames, rotations,
equivariance of the local-frame blocks) and the CUDA kernels on GPU (forward
and backward against the FP64 oracle MLP, training, SCF gain)."""
import os

import numpy as np
import pytest

import chinium_gb300 as cg
from chinium_gb300 import guess as G
from chinium_gb300 import molecules as M


def _rotation(seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1
    return q


def test_solid_harmonics_match_reference_tables():
    """The Helgaker-formula table reproduces the reference's explicit
    polynomials (AO/PureD.hpp:1-5, AO/PureF.hpp:1-7)."""
    p = np.random.default_rng(1).normal(size=(5, 3))
    x, y, z = p.T
    r2 = (p ** 2).sum(1)
    d = G.solid_harmonics(2, p)
    ref = [x * y * 3 ** 0.5, y * z * 3 ** 0.5, (3 * z * z - r2) / 2, x * z * 3 ** 0.5, (x * x - y * y) * 3 ** 0.5 / 2]
    assert np.allclose(d, ref)
    f = G.solid_harmonics(3, p)
    assert np.allclose(f[0], y * (3 * x * x - y * y) * 10 ** 0.5 / 4)
    assert np.allclose(f[3], (5 * z ** 3 - 3 * z * r2) / 2)


@pytest.mark.parametrize("t", [0, 1, -2, -3])
def test_shell_rotation_is_orthogonal_representation(t):
    Q1, Q2 = _rotation(1), _rotation(2)
    U1, U2 = G.shell_rotation(t, Q1), G.shell_rotation(t, Q2)
    assert np.allclose(U1 @ U1.T, np.eye(len(U1)), atol=1e-10)
    # composition: S(Q2^T Q1^T r) = U(Q1 Q2) S(r) = U2 U1 S(r)
    assert np.allclose(G.shell_rotation(t, Q1 @ Q2), U2 @ U1, atol=1e-10)


def test_local_blocks_are_rotation_invariant():
    """Rotating the molecule (and its density accordingly) leaves every
    local-frame block and feature vector unchanged."""
    Z, xyz = M.water_cluster(3, np.random.default_rng(4))
    basis = cg.Basis(Z, xyz, "def2-svp")
    n = basis.nbasis
    A = np.random.default_rng(5).normal(size=(n, n))
    D = A + A.T
    R = _rotation(9)
    xyz_r = xyz @ R.T
    types, first, count = G.atom_functions(basis)
    W = np.zeros((n, n))
    for a in range(len(Z)):
        W[first[a]:first[a] + count[a], first[a]:first[a] + count[a]] = G.atom_rotation(types[a], R)
    D_r = W.T @ D @ W
    X0, T0, M0 = G.dataset(Z, xyz, basis, D)
    X1, T1, M1 = G.dataset(Z, xyz_r, cg.Basis(Z, xyz_r, "def2-svp"), D_r)
    assert np.allclose(X0, X1, atol=1e-5)
    assert np.allclose(T0, T1, atol=1e-8)


@pytest.mark.gpu
def test_mlp_forward_backward_match_oracle():
    if not _gpu():
        pytest.skip("needs a GPU")
    from oracle import mlp_oracle as MO
    model = G.PairMLP(nin=9, hidden=32, layers=3, nout=7, seed=3)
    p = model.params()
    dims = [9, 32, 32, 32, 7]
    rng = np.random.default_rng(0)
    X = rng.normal(size=(50, 9)).astype(np.float32)
    Y = model.forward(X)
    Yo, _ = MO.forward(p, dims, X)
    assert np.allclose(Y, Yo, rtol=1e-4, atol=1e-5)
    dY = rng.normal(size=(50, 7)).astype(np.float32)
    g = model.grad(X, dY)
    go = MO.backward(p, dims, X, dY)
    assert np.allclose(g, go, rtol=1e-3, atol=1e-4 * np.abs(go).max())
    Yb = model.forward(X, bf16=True)
    assert np.abs(Yb - Yo).max() < 3e-2 * np.abs(Yo).max()


def _bf16_round(p):
    """FP32 -> nearest BF16 (ties to even), returned as FP64."""
    u = np.asarray(p, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


@pytest.mark.gpu
def test_mlp_tensor_core_products_at_network_shape():
    """The production network (79 -> 256 x 3 -> 196) on a ragged batch of
    1000 pairs: every dimension off the 128 x 64 tiles.  Training products
    (three BF16 planes each side) match FP64 to FP32 rounding; inference
    (BF16 weights, FP32 activations) matches an FP64 network whose weights
    are rounded to BF16, so the only error left is FP32 accumulation."""
    if not _gpu():
        pytest.skip("needs a GPU")
    from oracle import mlp_oracle as MO
    model = G.PairMLP(seed=5)
    dims = [model.nin] + [model.hidden] * model.layers + [model.nout]
    rng = np.random.default_rng(7)
    p = model.params()
    o = 0
    for fi, fo in zip(dims[:-1], dims[1:]):  # non-zero biases
        o += fi * fo
        p[o:o + fo] = 0.1 * rng.normal(size=fo)
        o += fo
    model.set_params(p)
    p = p.astype(np.float64)
    X = rng.normal(size=(1000, model.nin)).astype(np.float32)
    Yo, _ = MO.forward(p, dims, X)
    scale = np.abs(Yo).max()
    Y = model.forward(X)
    assert np.abs(Y - Yo).max() <= 2e-5 * scale, np.abs(Y - Yo).max() / scale
    dY = rng.normal(size=Yo.shape).astype(np.float32)
    g = model.grad(X, dY)
    go = MO.backward(p, dims, X, dY)
    assert np.abs(g - go).max() <= 2e-5 * np.abs(go).max(), np.abs(g - go).max() / np.abs(go).max()
    # inference: weights to BF16, biases stay FP32
    pb = p.copy()
    o = 0
    for fi, fo in zip(dims[:-1], dims[1:]):
        pb[o:o + fi * fo] = _bf16_round(p[o:o + fi * fo])
        o += fi * fo + fo
    Ybo, _ = MO.forward(pb, dims, X)
    Yb = model.forward(X, bf16=True)
    assert np.abs(Yb - Ybo).max() <= 2e-5 * scale, np.abs(Yb - Ybo).max() / scale
    assert np.abs(Yb - Yo).max() > 10 * np.abs(Yb - Ybo).max()  # BF16 weights do differ from FP32


@pytest.mark.gpu
def test_mlp_training_reduces_loss():
    if not _gpu():
        pytest.skip("needs a GPU")
    model = G.PairMLP(nin=9, hidden=64, layers=3, nout=4, seed=1)
    rng = np.random.default_rng(2)
    X = rng.normal(size=(512, 9)).astype(np.float32)
    T = np.stack([np.sin(X[:, 0]), X[:, 1] * X[:, 2], np.cos(X[:, 3] + X[:, 4]), X[:, 5] ** 2], axis=1).astype(np.float32)
    M_ = np.ones_like(T)
    l0 = model.train_step(X, T, M_, 1e-3)
    for _ in range(300):
        l = model.train_step(X, T, M_, 1e-3)
    assert l < 0.2 * l0


def _gpu():
    from conftest import has_gpu
    return has_gpu()


@pytest.mark.gpu
def test_learned_guess_reduces_scf_iterations():
    """The trained network (package weights) against the SAP guess on
    held-out water clusters (seeds disjoint from the training set)."""
    if not os.path.exists(G.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights in the package")
    from chinium_gb300.scf import run_scf
    model = G.load(G.DEFAULT_WEIGHTS)
    mols = M.water_clusters(4, seed=987654, kmin=2, kmax=3)
    it_sap, it_ml = [], []
    for Z, xyz in mols:
        r_sap = run_scf(Z, xyz, functional="PBE", guess="sap")
        ctx = r_sap.context
        D0 = G.guess_density(model, Z, xyz, ctx)
        r_ml = run_scf(Z, xyz, functional="PBE", guess=D0, context=ctx)
        assert r_sap.converged and r_ml.converged
        assert abs(r_ml.energy - r_sap.energy) < 1e-7
        it_sap.append(r_sap.iterations)
        it_ml.append(r_ml.iterations)
    print("iterations SAP", it_sap, "learned", it_ml)
    assert np.mean(it_ml) < np.mean(it_sap)


def test_batched_frames_and_features_match_per_pair():
    Z, xyz = M.water_cluster(5, np.random.default_rng(11))
    pr = G.pairs(xyz)
    Qs, X = G.frames_and_features(Z, xyz, pr)
    for p in range(0, len(pr), 7):
        a, b = pr[p]
        Q = G.pair_frame(xyz, a, b)
        assert np.allclose(Qs[p], Q, atol=1e-12)
        assert np.allclose(X[p], G.pair_features(Z, xyz, a, b, Q), atol=1e-6)
    # a lone atom has an identity frame
    Qs1, X1 = G.frames_and_features([8], np.zeros((1, 3)), [(0, 0)])
    assert np.allclose(Qs1[0], np.eye(3)) and np.allclose(Qs1[0], G.pair_frame(np.zeros((1, 3)), 0, 0))


@pytest.mark.gpu
def test_learned_guess_with_sap_fallback_in_scf():
    """guess="learned" in the SCF driver: the network inside its scope, the
    SAP guess outside it and when the learned start does not converge."""
    from chinium_gb300.scf import run_scf
    Z, xyz = M.water_cluster(3, np.random.default_rng(77))
    r = run_scf(Z, xyz, functional="PBE", guess="learned")
    assert r.converged and r.guess_used == "learned"
    ref = run_scf(Z, xyz, functional="PBE", guess="sap", context=r.context)
    assert abs(r.energy - ref.energy) < 1e-7
    Zm, xm = M.alkane(1, np.random.default_rng(0))  # methane: carbon is outside the model
    rm = run_scf(Zm, xm, functional="PBE", guess="learned")
    assert rm.converged and rm.guess_used.startswith("sap")
    rf = run_scf(Z, xyz, functional="PBE", guess="learned", max_iter=4, context=r.context)
    assert rf.guess_used.startswith("sap (learned start did not converge")


def test_batched_block_assembly_matches_per_pair_loop():
    """assemble_blocks (one batched product per block layout) against the
    per-pair rotation and placement it replaces."""
    rng = np.random.default_rng(11)
    count = [14, 5, 5, 14, 5]
    first = list(np.cumsum([0] + count[:-1]))
    n = sum(count)
    pr = [(a, b) for a in range(5) for b in range(a, 5)]
    Y = rng.normal(size=(len(pr), G.MAX_FUNC, G.MAX_FUNC)).astype(np.float32)
    Uas = [np.linalg.qr(rng.normal(size=(count[a], count[a])))[0] for a, _ in pr]
    Ubs = [np.linalg.qr(rng.normal(size=(count[b], count[b])))[0] for _, b in pr]
    want = np.zeros((n, n))
    for (a, b), Ua, Ub, y in zip(pr, Uas, Ubs, Y):
        blk = Ua.T @ y[:count[a], :count[b]].astype(np.float64) @ Ub
        want[first[a]:first[a] + count[a], first[b]:first[b] + count[b]] = blk
        if a != b:
            want[first[b]:first[b] + count[b], first[a]:first[a] + count[a]] = blk.T
    got = G.assemble_blocks(pr, Y, Uas, Ubs, first, count, n)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)


def test_overlap_metric():
    from chinium_gb300.scf import overlap_metric
    rng = np.random.default_rng(2)
    A = rng.normal(size=(9, 9))
    S = A @ A.T + 9 * np.eye(9)
    ctx = {}
    X, Xh, Sh = overlap_metric(S, ctx)
    np.testing.assert_allclose(X.T @ S @ X, np.eye(9), atol=1e-12)
    np.testing.assert_allclose(Xh @ S @ Xh, np.eye(9), atol=1e-12)
    np.testing.assert_allclose(Sh @ Sh, S, atol=1e-11)
    assert overlap_metric(S, ctx)[0] is X
