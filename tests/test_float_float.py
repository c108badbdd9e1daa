"""The float-float scalar of the functional library (xcf::ff in
chinium_gb300/csrc/functional.cuh: Dekker/Knuth error-free sums and
products, exp by argument reduction and an expm1 series, log/sqrt/cbrt by a
Newton step) on the host, compiled from the same header with g++
(tests/ff_check.cpp), against numpy's FP64: the arithmetic the mixed path's
energy density runs on the FP32 pipe.  CPU only."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "chinium_gb300", "csrc")


@pytest.fixture(scope="module")
def ff_check(tmp_path_factory):
    gxx = shutil.which("g++")
    inc = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(inc):
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("ff") / "ff_check")
    r = subprocess.run([gxx, "-O2", "-std=c++17", "-I" + CSRC, "-I" + inc, os.path.join(HERE, "ff_check.cpp"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def run(op, x, y=None):
        y = np.zeros_like(x) if y is None else y
        inp = "".join("%s %.17g %.17g\n" % (op, a, b) for a, b in zip(x, y))
        out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout
        return np.array([float(v) for v in out.split()])
    return run


def ff_round(x):
    """x as the float-float pair the library forms from a double (hi + lo)."""
    hi = x.astype(np.float32).astype(np.float64)
    return hi + (x - hi).astype(np.float32).astype(np.float64)


rng = np.random.default_rng(0)
X = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), 400)) * rng.choice([-1.0, 1.0], 400)
Y = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), 400)) * rng.choice([-1.0, 1.0], 400)


def test_representation_keeps_48_bits(ff_check):
    got = ff_check("split", X)
    assert np.all(np.abs(got - X) <= 2.0 ** -47 * np.abs(X))
    assert np.array_equal(got, ff_round(X))


@pytest.mark.parametrize("op,f", [("add", np.add), ("sub", np.subtract), ("mul", np.multiply),
                                  ("div", np.divide)])
def test_arithmetic(ff_check, op, f):
    a, b = ff_round(X), ff_round(Y)
    got = ff_check(op, X, Y)
    ref = f(a, b)
    # sums: relative to the larger operand (cancellation); products, quotients: relative
    scale = np.maximum(np.abs(a), np.abs(b)) if op in ("add", "sub") else np.abs(ref)
    assert np.all(np.abs(got - ref) <= 1e-14 * scale), np.max(np.abs(got - ref) / scale)


def test_exp(ff_check):
    # results whose lo part stays a normal float (the functionals' arguments are within)
    x = np.concatenate([rng.uniform(-60, 80, 300), [0.0, 1e-9, -1e-9, 0.5, -0.5, 30.0, -30.0]])
    got = ff_check("exp", x)
    ref = np.exp(ff_round(x))
    assert np.all(np.abs(got - ref) <= 4e-14 * ref), np.max(np.abs(got - ref) / ref)
    # below FP32's range the result is 0 (the functionals' exp arguments there are negative)
    assert np.all(ff_check("exp", np.array([-90.0, -300.0])) == 0.0)


def test_log(ff_check):
    x = np.exp(rng.uniform(np.log(1e-30), np.log(1e30), 300))
    got = ff_check("log", x)
    ref = np.log(ff_round(x))
    assert np.all(np.abs(got - ref) <= 1e-14 * np.maximum(1.0, np.abs(ref))), np.max(np.abs(got - ref))


@pytest.mark.parametrize("op,f", [("sqrt", np.sqrt), ("cbrt", np.cbrt)])
def test_roots(ff_check, op, f):
    """One Newton step from the FP32 root: error ~ (FP32 error)^2, ~1.4e-14 at most."""
    x = np.exp(rng.uniform(np.log(1e-30), np.log(1e30), 300))
    got = ff_check(op, x)
    ref = f(ff_round(x))
    assert np.all(np.abs(got - ref) <= 3e-14 * ref), np.max(np.abs(got - ref) / ref)


@pytest.mark.parametrize("k", [-11, -4, -1, 1, 2, 4, 5, 8])
def test_thirds(ff_check, k):
    """x^(k/3) as the functionals take every power (pow3: cbrt, then binary powering)."""
    x = np.exp(rng.uniform(np.log(1e-8), np.log(1e3), 200))
    got = ff_check("pow3", x, np.full_like(x, k))
    ref = np.cbrt(ff_round(x)) ** k
    # the cube root's error times |k|, plus the powering's roundings
    assert np.all(np.abs(got - ref) <= 3e-13 * ref), np.max(np.abs(got - ref) / ref)
