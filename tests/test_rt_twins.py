"""aether::rt (include/aether/rt.h; expr/Rt.h): the rolled-loop twins of the
per-sample reductions and contractions return the bits of the static forms
they stand in for (tests/cpp/rt_twins.cpp): dot, sum, the norm family,
maxNorm, isFinite, matDot, matVec (=, +=, -=), matMat, transposed operands and
store, over Items and per-sample proxies, 144-element and 8x40 operands
included. Contraction is off in every build (the device code and the host
code of the nvcc build too: an aarch64 host compiler contracts by default),
so equal means bit-equal.

CPU: the host build. GPU: the same checks, one sample per thread."""

import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
SRC = os.path.join(REPO, "tests", "cpp", "rt_twins.cpp")


def _run(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "rt twins ok" in r.stdout, r.stdout + r.stderr


def test_twins_on_the_host(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "rt_twins")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-ffp-contract=off", "-Wall", "-Wextra", "-I", INCLUDE, SRC, "-o",
                        exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _run(exe)


def _nvcc(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "rt_twins_cu")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "--fmad=false", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, SRC, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_twins_compile_for_sm103a(tmp_path):
    _nvcc(tmp_path)


@pytest.mark.gpu
def test_twins_in_a_kernel(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _run(_nvcc(tmp_path))
