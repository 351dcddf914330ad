"""reshaped<Ms...> (include/aether/reshape.h; view/Reshape.h),
copyAsync(View, View, Stream) (include/aether/view_copy.h; view/Copy.h) and
accum::AppendCounter (include/aether/append_counter.h;
accum/AppendCounter.h), through tests/cpp/view_tools.cpp: the reference's
reshape, view-copy and append-counter rows.

CPU: reshapes of host views and the append counter's logic over host words
(sequential, eight racing threads, overflow), under the sanitizers; the device
program compiled for sm_103a. GPU: copies between device and page-locked
views with their refusals, and kernels appending into an Array's spare
capacity within and past it."""

import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(REPO, "aether_gb300", "lib")
SRC = os.path.join(REPO, "tests", "cpp", "view_tools.cpp")


def _run(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "view tools ok" in r.stdout, r.stdout + r.stderr


def test_host_cases(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    probe = subprocess.run([cxx, "-fsanitize=address,undefined", "-x", "c++", "-", "-o", str(tmp_path / "p")],
                           input="int main(){}", capture_output=True, text=True)
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"] if probe.returncode == 0 else []
    exe = str(tmp_path / "view_tools")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-g", "-Wall", "-Wextra", "-pthread", "-I", INCLUDE, SRC, "-o", exe]
                       + san, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _run(exe)


def _nvcc(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    if not os.path.exists(os.path.join(LIBDIR, "libaether_gb300.so")):
        pytest.skip("engine library not built")
    exe = str(tmp_path / "view_tools_cu")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "-I", INCLUDE, SRC, "-o", exe, "-L", LIBDIR, "-laether_gb300", "-Xlinker", "-rpath," + LIBDIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_device_program_builds(tmp_path):
    _nvcc(tmp_path)


@pytest.mark.gpu
def test_device_cases(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import aether_gb300  # noqa: F401  (the engine library is built)
    _run(_nvcc(tmp_path))
