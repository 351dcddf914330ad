"""aether::Chunk, copy, copyAsync, fill and make_view(chunk)
(include/aether/chunk.h; chunk/Chunk.h, chunk/Copy.h, chunk/Fill.h) through
tests/cpp/chunk_api.cpp: ownership and moves, borrowed bytes, host copies and
fills, views over chunks, and the refusals (size mismatch, a direct
host<->device pair checked before the empty case, asynchronous copies of
pageable memory, fill widths, alignment).

CPU: the host cases against the engine library, under the sanitizers.
GPU: device and page-locked chunks, stream-ordered allocation, copies both
ways and a patterned device fill."""

import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(REPO, "aether_gb300", "lib")
SRC = os.path.join(REPO, "tests", "cpp", "chunk_api.cpp")


def _lib():
    if not os.path.exists(os.path.join(LIBDIR, "libaether_gb300.so")):
        pytest.skip("engine library not built")


def _run(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "chunk ok" in r.stdout, r.stdout + r.stderr


def test_host_cases(tmp_path):
    _lib()
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    probe = subprocess.run([cxx, "-fsanitize=address,undefined", "-x", "c++", "-", "-o", str(tmp_path / "p")],
                           input="int main(){}", capture_output=True, text=True)
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"] if probe.returncode == 0 else []
    exe = str(tmp_path / "chunk_api")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-g", "-Wall", "-Wextra", "-I", INCLUDE, SRC, "-o", exe, "-L",
                        LIBDIR, "-laether_gb300", "-Wl,-rpath," + LIBDIR] + san, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _run(exe)


def _nvcc(tmp_path):
    _lib()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "chunk_api_cu")
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
