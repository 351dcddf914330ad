"""aether::math, the whole facade (math/math.h and its family headers), on the
host and in a device kernel over one corpus (tests/cpp/math_facade.cpp).

* CPU: the host results are std::'s (the facade routes there), and the
  reference-specific semantics hold: round half away from zero, rint half to
  even, numpy's floored remainder (the divisor's sign, signed zeros
  included), sign(0) = sign(NaN) = 0, clip letting NaN through.
* GPU: exact operations (rounding, fmod, fdim, copysign, min/max, sign,
  clip, remainder, the predicates, sqrt, rsqrt, abs) bit for bit against the
  host; transcendentals within the reference's own device-versus-host ulp
  table (tests/test_MathParity_common.h:229-250: 2 for expm1, log1p, cosh,
  exp2, log2, log10, hypot, 3 for sinh, atanh, erf, pow, 4 for asinh, acosh,
  cbrt, 6 for erfc), 3 for the trigonometric and inverse trigonometric
  functions and 2 for the rest (CUDA's documented bounds plus glibc's own).
"""

import math
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
SRC = os.path.join(REPO, "tests", "cpp", "math_facade.cpp")
KN, KFNS = 512, 43
NAMES = ["sqrt", "rsqrt", "exp", "log", "log1p", "sin", "cos", "cbrt", "exp2", "expm1", "log2", "log10", "tan",
         "asin", "acos", "atan", "sinh", "cosh", "tanh", "erf", "abs", "floor", "ceil", "trunc", "round", "rint",
         "asinh", "acosh", "atanh", "erfc", "exp10", "pow", "atan2", "hypot", "min", "max", "fmod", "fdim",
         "copysign", "remainder", "sign", "clip", "predicates"]
EXACT = {"sqrt", "rsqrt", "abs", "floor", "ceil", "trunc", "round", "rint", "min", "max", "fmod", "fdim", "copysign",
         "remainder", "sign", "clip", "predicates"}
ULPS = {"expm1": 2, "log1p": 2, "cosh": 2, "exp2": 2, "log2": 2, "log10": 2, "hypot": 2, "sinh": 3, "atanh": 3,
        "erf": 3, "pow": 3, "asinh": 4, "acosh": 4, "cbrt": 4, "erfc": 6,
        # CUDA's documented bounds plus glibc's (the native parity tests' table)
        "sin": 3, "cos": 3, "tan": 3, "asin": 3, "acos": 3, "atan": 3, "atan2": 3}


def corpus():
    sp = [0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.5, -2.5, 1e-300, 3.0, 1e300, -7.75]
    x = np.array([sp[i] if i < 12 else -12.0 + 24.0 * i / KN for i in range(KN)])
    y = np.array([(0.25 + 2.75 * ((i * 37) % KN) / KN) * (-1 if i % 3 == 0 else 1) for i in range(KN)])
    return x, y


def run(exe, tmp_path):
    out = tmp_path / (os.path.basename(exe) + ".bin")
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "math facade ok" in r.stdout, r.stdout + r.stderr
    return np.fromfile(str(out), dtype=np.float64).reshape(KFNS, KN)


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("facade")
    exe = str(d / "math_facade")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-I", INCLUDE, SRC, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return run(exe, d)


def test_host_semantics(host):
    x, y = corpus()
    got = dict(zip(NAMES, host))
    assert np.array_equal(got["round"], np.where(np.abs(x - np.trunc(x)) == 0.5, np.trunc(x) + np.sign(x), np.round(x)))
    assert np.array_equal(got["rint"], np.rint(x))
    # numpy's remainder: the divisor's sign, zeros included
    ref = np.remainder(x, y)
    assert np.array_equal(got["remainder"], ref)
    assert np.array_equal(np.signbit(got["remainder"]), np.signbit(ref))
    assert np.array_equal(got["fmod"], np.fmod(x, y))
    assert np.array_equal(got["sign"], np.sign(x))
    clip_ref = np.where(x >= -1.0, x, -1.0)
    clip_ref = np.where(clip_ref <= y, clip_ref, y)
    assert np.array_equal(got["clip"], clip_ref)
    assert np.array_equal(got["copysign"], np.copysign(x, y))
    assert np.array_equal(got["fdim"], np.where(x > y, x - y, 0.0))
    assert got["exp10"][20] == pytest.approx(10.0 ** np.clip(x[20], -12, 12), rel=1e-15)
    assert np.allclose(got["asinh"], np.arcsinh(x), rtol=1e-15, atol=0)
    assert all(math.isclose(a, math.erfc(b), rel_tol=1e-15, abs_tol=1e-300) for a, b in zip(got["erfc"], x))


def test_facade_compiles_for_sm103a(tmp_path):
    _nvcc(tmp_path)


def _nvcc(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "math_facade_cu")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "--fmad=false", "-I", INCLUDE, SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def ulp_dist(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    same = (a == b) | both_nan
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    ia = np.where(ia < 0, np.int64(-0x8000000000000000) - ia, ia)
    ib = np.where(ib < 0, np.int64(-0x8000000000000000) - ib, ib)
    d = np.abs(ia - ib)
    return np.where(same, 0, d)


@pytest.mark.gpu
def test_device_matches_host(tmp_path, host):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = run(_nvcc(tmp_path), tmp_path)
    for k, name in enumerate(NAMES):
        if name in EXACT:
            assert np.array_equal(dev[k], host[k], equal_nan=True), name
        else:
            assert int(ulp_dist(dev[k], host[k]).max()) <= ULPS.get(name, 2), name
