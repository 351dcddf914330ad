"""aether::random's whole leaf API against the reference's own draws.

tests/cpp/random_leaves.cpp draws, through include/aether, the cases the
reference driver (oracle/ref_driver.cpp) draws through the reference's
headers into tests/golden/ref_cases.npz: per-component Item parameters of
normal, lognormal, exponential and bernoulli; uniformInt in 32 and 64 bits;
multivariateNormal from cholesky in double and float; the free-function
spelling; and the index-free get<I>() draws (random/detail/
DistributionLeaf.h, MultivariateNormalLeaf.h, LowerTriangular.h, free.h).

* CPU: compiled by g++ with contraction off, every value equals the
  reference's bit for bit.
* GPU: the same source compiled by nvcc (--fmad=false) draws one sample per
  thread: integer, uniform and bernoulli draws bit-exact; draws through
  CUDA's log, exp, sqrt and sin within the reference's own device-versus-host
  tolerance for normals, 1e-12 abs+rel in double and 1e-5 in float
  (tests/random/golden_random.h:437-441).
"""

import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
SRC = os.path.join(REPO, "tests", "cpp", "random_leaves.cpp")
N = 1000

# (golden name, planes of the f64 block) in the program's output order
F64_PLANES = [("leafi_normal", 0, 3), ("leafi_lognormal", 3, 6), ("leafi_exponential", 6, 9),
              ("leafi_bernoulli", 9, 12), ("leaf_mvn", 12, 15), ("free_uniform", 15, 17),
              ("free_seed_normal", 17, 19)]
EXACT_F64 = {"leafi_bernoulli", "free_uniform"}
# index-free entries drawn without a transcendental function
INDEX_FREE_EXACT = [0, 1, 2, 8, 9, 10, 11, 15]
INDEX_FREE_FLOAT = [3, 4, 14]

DOUBLE_TOL = 1e-12
FLOAT_TOL = 1e-5


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(REPO, "tests", "golden", "ref_cases.npz"))


def read_output(path, n):
    raw = open(path, "rb").read()
    off = 0
    out = {}

    def take(dt, count):
        nonlocal off
        a = np.frombuffer(raw, dtype=dt, count=count, offset=off)
        off += a.nbytes
        return a

    f = take(np.float64, 19 * n).reshape(19, n)
    for name, lo, hi in F64_PLANES:
        out[name] = f[lo:hi]
    out["index_free"] = take(np.float64, 16)[None]
    out["leaf_uniform_int"] = take(np.int32, 3 * n).reshape(3, n)
    out["leaf_uniform_int64"] = take(np.int64, 2 * n).reshape(2, n)
    out["leaf_mvn_f32"] = take(np.float32, 2 * n).reshape(2, n)
    out["mvn_cholesky"] = take(np.float64, 6)[None]
    assert off == len(raw)
    return out


def run(exe, tmp_path):
    out = tmp_path / "leaves.bin"
    r = subprocess.run([exe, str(out), str(N)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "random leaves ok" in r.stdout, r.stdout + r.stderr
    return read_output(str(out), N)


def abs_rel(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.max(np.abs(got - ref) / (1.0 + np.abs(ref))))


def test_golden_holds_the_new_cases(golden):
    for name in [p[0] for p in F64_PLANES] + ["index_free", "leaf_uniform_int", "leaf_uniform_int64",
                                              "leaf_mvn_f32", "mvn_cholesky"]:
        assert name in golden.files, name
    ints = golden["leaf_uniform_int"]
    assert ints.min() >= -5 and ints.max() <= 17 and len(np.unique(ints)) == 23
    big = golden["leaf_uniform_int64"]
    assert big.min() >= -(1 << 40) and big.max() <= (1 << 41)
    assert set(np.unique(golden["leafi_bernoulli"])) <= {0.0, 1.0}


def test_host_draws_are_the_references(tmp_path, golden):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "random_leaves")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-I", INCLUDE, SRC, "-o",
                        exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = run(exe, tmp_path)
    for name, a in got.items():
        assert a.dtype == golden[name].dtype, name
        assert np.array_equal(a, golden[name]), name


def _nvcc(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "random_leaves_cu")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "--fmad=false", "-I", INCLUDE, SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_leaves_compile_for_sm103a(tmp_path):
    _nvcc(tmp_path)


@pytest.mark.gpu
def test_device_draws_match_the_references(tmp_path, golden):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    got = run(_nvcc(tmp_path), tmp_path)
    for name in ("leaf_uniform_int", "leaf_uniform_int64", "mvn_cholesky"):
        assert np.array_equal(got[name], golden[name]), name
    for name, _, _ in F64_PLANES:
        if name in EXACT_F64:
            assert np.array_equal(got[name], golden[name]), name
        else:
            assert abs_rel(got[name], golden[name]) <= DOUBLE_TOL, name
    assert abs_rel(got["leaf_mvn_f32"], golden["leaf_mvn_f32"]) <= FLOAT_TOL
    g, r = got["index_free"][0], golden["index_free"][0]
    assert np.array_equal(g[INDEX_FREE_EXACT], r[INDEX_FREE_EXACT])
    rest = [k for k in range(16) if k not in INDEX_FREE_EXACT]
    for k in rest:
        tol = FLOAT_TOL if k in INDEX_FREE_FLOAT else DOUBLE_TOL
        assert abs_rel(g[k], r[k]) <= tol, k
