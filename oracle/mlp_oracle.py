"""ORACLE -- test infrastructure only.  FP64 numpy restatement of the
per-atom-pair MLP (include/chinium_guess.h): x -> [Linear, SiLU] x L ->
Linear, parameters flat per layer (W fan_in x fan_out row-major, then b).
Used to check the CUDA forward and backward kernels."""
import numpy as np


def unpack(p, dims):
    out, o = [], 0
    for fi, fo in zip(dims[:-1], dims[1:]):
        W = p[o:o + fi * fo].reshape(fi, fo)
        o += fi * fo
        b = p[o:o + fo]
        o += fo
        out.append((W, b))
    return out


def silu(z):
    return z / (1 + np.exp(-z))


def dsilu(z):
    s = 1 / (1 + np.exp(-z))
    return s * (1 + z * (1 - s))


def forward(p, dims, X):
    layers = unpack(np.asarray(p, dtype=np.float64), dims)
    h = np.asarray(X, dtype=np.float64)
    cache = []
    for i, (W, b) in enumerate(layers):
        z = h @ W + b
        cache.append((h, z))
        h = silu(z) if i < len(layers) - 1 else z
    return h, cache


def backward(p, dims, X, dY):
    """Gradient of sum(dY * net(X)) with respect to p (flat, same layout)."""
    layers = unpack(np.asarray(p, dtype=np.float64), dims)
    _, cache = forward(p, dims, X)
    grads = []
    d = np.asarray(dY, dtype=np.float64)
    for i in range(len(layers) - 1, -1, -1):
        W, _ = layers[i]
        h, z = cache[i]
        dz = d if i == len(layers) - 1 else d * dsilu(z)
        grads.append((h.T @ dz, dz.sum(0)))
        d = dz @ W.T
    grads.reverse()
    return np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
