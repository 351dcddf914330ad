"""aether::accum::atomic (include/aether/accum_atomic.h; accum/atomic.h):
the magnitude minimum that keeps the stored sign, the integer maximum,
monotone one-byte bool slots and the compensated sum, under 16384 concurrent
writers (tests/cpp/accum_atomic.cpp; the reference's tests/test_Atomic).

CPU: eight host threads, under the sanitizers. GPU: one kernel of 64 blocks
of 256 threads."""

import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
SRC = os.path.join(REPO, "tests", "cpp", "accum_atomic.cpp")


def _run(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "atomic ok" in r.stdout, r.stdout + r.stderr


def test_host_threads(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    probe = subprocess.run([cxx, "-fsanitize=address,undefined", "-x", "c++", "-", "-o", str(tmp_path / "p")],
                           input="int main(){}", capture_output=True, text=True)
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"] if probe.returncode == 0 else []
    exe = str(tmp_path / "accum_atomic")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-g", "-Wall", "-Wextra", "-pthread", "-I", INCLUDE, SRC, "-o", exe]
                       + san, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _run(exe)


def _nvcc(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "accum_atomic_cu")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "-I", INCLUDE, SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_compiles_for_sm103a(tmp_path):
    _nvcc(tmp_path)


@pytest.mark.gpu
def test_device_writers(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _run(_nvcc(tmp_path))
