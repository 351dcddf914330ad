"""The per-sample expression surface on Items (tests/cpp/expr_surface.cpp):
the reference's expression-depth, structural, reduction and rank-0 item rows
(tests/test_ExprDepth.cpp, test_ExprStructural, test_ExprReduce,
test_ItemRank0) and the Item factories (view/Item.h:195-225), run on the host
by a host compiler and in a kernel on the device."""

import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
SRC = os.path.join(REPO, "tests", "cpp", "expr_surface.cpp")


def _run(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "expr surface ok" in r.stdout, r.stdout + r.stderr


def test_surface_on_the_host(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "expr_surface")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", INCLUDE, SRC, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _run(exe)


def _nvcc(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "expr_surface_cu")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "-I", INCLUDE, SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_surface_compiles_for_sm103a(tmp_path):
    _nvcc(tmp_path)


@pytest.mark.gpu
def test_surface_in_a_kernel(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _run(_nvcc(tmp_path))
