"""The functional library the CUDA kernels run (chinium_gb300/csrc/
functional.cuh: published formulas, potentials by forward-mode dual numbers)
compiled for the host with g++ (tests/xc_point_check.cpp) and checked on the
CPU: against the oracle's independent restatement (complex-step potentials)
on random points of every configured id set, restricted and unrestricted,
and against the hydrogen-atom values of tests/test_functional_pins.py.  The
same source runs on the GPU (tests/test_gpu_parity.py compares the device
results with the oracle).  CPU only."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "chinium_gb300", "csrc")

ID_SETS = [[1], [1, 7], [8], [106], [131], [101, 130], [321, 322], [402], [406], [436], [202, 231], [457],
           [497, 498]]


@pytest.fixture(scope="module")
def xc_host(tmp_path_factory):
    gxx = shutil.which("g++")
    inc = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(inc):
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("xc") / "xc_point_check")
    r = subprocess.run([gxx, "-O2", "-std=c++17", "-I" + CSRC, "-I" + inc, os.path.join(HERE, "xc_point_check.cpp"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def run(ids, ns, inputs, mode="v"):
        """mode "v": inputs (npoints, 3) restricted or (npoints, 7)
        unrestricted; returns eps (npoints,) and dv (npoints, 3 or 7).
        mode "f" (LDA / GGA): inputs (npoints, 2) or (npoints, 5); returns
        eps and the potentials followed by the second derivatives."""
        head = "%s %d %d %s" % (mode, ns, len(ids), " ".join(str(i) for i in ids))
        text = "".join(head + " " + " ".join("%.17g" % v for v in row) + "\n" for row in inputs)
        out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout
        vals = np.array([[float(v) for v in line.split()] for line in out.strip().splitlines()])
        return vals[:, 0], vals[:, 1:]
    return run


def random_points(ns, n, rng):
    """Densities over 9 decades, reduced gradients and kinetic energy
    densities above the von Weizsaecker bound (the region of molecules)."""
    if ns == 1:
        rho = 10 ** rng.uniform(-6, 3, n)
        sig = rho ** (8 / 3) * 10 ** rng.uniform(-4, 1.5, n)
        tau = sig / (8 * rho) * (1 + 10 ** rng.uniform(-4, 1, n))
        return np.stack([rho, sig, tau], axis=1)
    ra = 10 ** rng.uniform(-6, 3, n)
    rb = ra * 10 ** rng.uniform(-3, 0.5, n)
    saa = ra ** (8 / 3) * 10 ** rng.uniform(-4, 1.5, n)
    sbb = rb ** (8 / 3) * 10 ** rng.uniform(-4, 1.5, n)
    sab = np.sqrt(saa * sbb) * rng.uniform(-1, 1, n)
    ta = saa / (8 * ra) * (1 + 10 ** rng.uniform(-4, 1, n))
    tb = sbb / (8 * rb) * (1 + 10 ** rng.uniform(-4, 1, n))
    return np.stack([ra, rb, saa, sab, sbb, ta, tb], axis=1)


@pytest.mark.parametrize("ns", [1, 2])
@pytest.mark.parametrize("ids", ID_SETS, ids=lambda s: "+".join(map(str, s)))
def test_library_matches_the_oracle_on_points(xc_host, ids, ns):
    rng = np.random.default_rng(11)
    x = random_points(ns, 300, rng)
    eps, dv = xc_host(ids, ns, x)
    if ns == 1:
        ref = O.functional(ids, 1, x[:, 0], x[:, 1], x[:, 2])
    else:
        ref = O.functional(ids, 2, x[:, 0:2].T, x[:, 2:5].T, x[:, 5:7].T)
    fam = O.family(ids)
    # the scale of a sum over ids is the sum of its terms' magnitudes (PBE's
    # exchange and correlation v_sigma nearly cancel at some densities)
    parts = [O.functional([i], 1, x[:, 0], x[:, 1], x[:, 2]) if ns == 1 else
             O.functional([i], 2, x[:, 0:2].T, x[:, 2:5].T, x[:, 5:7].T) for i in ids]
    # library order: restricted (rho, sigma, tau); unrestricted (ra, rb, saa, sab, sbb, ta, tb)
    got = {"eps": eps[None, :],
           "vrho": dv[:, 0:ns].T,
           "vsigma": dv[:, ns:ns + (1 if ns == 1 else 3)].T,
           "vtau": dv[:, (2 if ns == 1 else 5):].T}
    for k, name in enumerate(["eps", "vrho", "vsigma", "vtau"]):
        if name == "vsigma" and fam < 1 or name == "vtau" and fam < 2:
            continue
        r = np.asarray(ref[k]).reshape(got[name].shape)
        q = got[name]
        mag = sum(np.abs(np.asarray(p[k]).reshape(q.shape)) for p in parts)
        err = np.abs(q - r) / (mag + 1e-12 * mag.max() + 1e-300)
        # same host libm on both sides: differences are the two derivative
        # methods' roundings and the formulas' cancellations
        assert np.quantile(err, 0.99) < 1e-10, (name, np.quantile(err, 0.99))
        assert err.max() < 1e-7, (name, err.max())


def moderate_points(ns, n, rng):
    """Densities 1e-3 .. 1e2 with ordinary reduced gradients: the region where
    the oracle's second derivatives (Richardson differences of its exact
    complex-step gradients) are accurate to ~1e-9."""
    if ns == 1:
        rho = 10 ** rng.uniform(-3, 2, n)
        return np.stack([rho, rho ** (8 / 3) * 10 ** rng.uniform(-2, 1, n)], axis=1)
    ra = 10 ** rng.uniform(-3, 2, n)
    rb = ra * 10 ** rng.uniform(-1, 0.5, n)
    saa = ra ** (8 / 3) * 10 ** rng.uniform(-2, 1, n)
    sbb = rb ** (8 / 3) * 10 ** rng.uniform(-2, 1, n)
    sab = np.sqrt(saa * sbb) * rng.uniform(-0.9, 0.9, n)
    return np.stack([ra, rb, saa, sab, sbb], axis=1)


# input index pairs of the second-derivative components (libxc layouts)
PAIRS = {1: [(0, 0), (0, 1), (1, 1)],
         2: [(0, 0), (0, 1), (1, 1)] + [(a, s) for a in (0, 1) for s in (2, 3, 4)] +
            [(2, 2), (2, 3), (2, 4), (3, 3), (3, 4), (4, 4)]}


@pytest.mark.parametrize("ns", [1, 2])
@pytest.mark.parametrize("ids", [i for i in ID_SETS if O.family(i) <= 1], ids=lambda s: "+".join(map(str, s)))
def test_library_second_derivatives_match_the_oracle(xc_host, ids, ns):
    """The response's kernel f_xc: second-derivative jets of the library
    against the oracle's, each component scaled by its two inputs
    (rho^2, rho sigma, sigma^2, ...) and compared with the energy density:
    a measure that also holds where a component vanishes identically (LYP is
    linear in the sigmas)."""
    rng = np.random.default_rng(12)
    inp = moderate_points(ns, 300, rng)
    _, out = xc_host(ids, ns, inp, mode="f")
    npot = 2 if ns == 1 else 5
    got = out[:, npot:].T  # (3 or 15, npoints)
    if ns == 1:
        ref = np.concatenate(O.functional_fxc(ids, 1, inp[:, 0], inp[:, 1]), axis=0)
        eden = sum(np.abs(O.functional([i], 1, inp[:, 0], inp[:, 1])[0].ravel()) for i in ids) * inp[:, 0]
    else:
        ref = np.concatenate(O.functional_fxc(ids, 2, inp[:, 0:2].T, inp[:, 2:5].T), axis=0)
        eden = sum(np.abs(O.functional([i], 2, inp[:, 0:2].T, inp[:, 2:5].T)[0].ravel()) for i in ids) * \
            (inp[:, 0] + inp[:, 1])
    u = np.abs(inp.T).copy()
    if ns == 2:
        u[3] = np.abs(inp[:, 3]) + np.sqrt(inp[:, 2] * inp[:, 4])  # sigma_ab's scale
    pairs = PAIRS[ns]
    if O.family(ids) == 0:  # LDA: v2rho2 only
        pairs = pairs[:1] if ns == 1 else pairs[:3]
    for k, (i, j) in enumerate(pairs):
        err = np.abs(got[k] - ref[k]) * u[i] * u[j] / eden
        # measured ~5e-13 at most
        assert np.quantile(err, 0.99) < 1e-11 and err.max() < 1e-10, (k, np.quantile(err, 0.99), err.max())


def _hydrogen():
    x, w = np.polynomial.legendre.leggauss(800)
    t = 0.5 * (x + 1.0)
    r = t / (1.0 - t)
    W = 4.0 * np.pi * r**2 * 0.5 * w / (1.0 - t) ** 2
    return W, np.exp(-2.0 * r) / np.pi


@pytest.mark.parametrize("ids,ref,tol", [
    ([1], -(81.0 / 512.0) * 3.0 ** (1 / 3) * 2.0 ** (4 / 3) * np.pi ** (-2 / 3), 1e-12),
    ([202], -5.0 / 16.0, 1e-6),
    ([497], -5.0 / 16.0, 5e-6),
    ([106], -0.3098, 5e-5),
    ([101], -0.3059, 5e-5),
    ([321], -0.3059, 5e-5),
])
def test_library_exchange_of_the_hydrogen_atom(xc_host, ids, ref, tol):
    """Spin scaling: E_x[rho, 0] = E_x[2 rho] / 2 through the restricted
    evaluation (density 2 rho, sigma 16 rho^2, tau rho)."""
    W, rho = _hydrogen()
    n = 2.0 * rho
    eps, _ = xc_host(ids, 1, np.stack([n, 16.0 * rho**2, rho], axis=1))
    ex = 0.5 * np.sum(W * n * eps)
    assert abs(ex - ref) < tol, ex


@pytest.mark.parametrize("ids,ref,tol", [([130], -0.0060, 5e-5), ([322], -0.0060, 5e-5), ([131], 0.0, 1e-10),
                                         ([231], 0.0, 1e-10), ([498], 0.0, 1e-10)])
def test_library_correlation_of_the_hydrogen_atom(xc_host, ids, ref, tol):
    W, rho = _hydrogen()
    z = np.zeros_like(rho)
    eps, _ = xc_host(ids, 2, np.stack([rho, z, 4.0 * rho**2, z, z, 0.5 * rho, z], axis=1))
    ec = np.sum(W * rho * eps)
    assert abs(ec - ref) < tol, ec
