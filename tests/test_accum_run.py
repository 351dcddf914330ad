"""aether::accum::run (include/aether/accum_run.h; accum/run.h): keyed
accumulation with one atomic per run of lanes sharing a slot
(tests/cpp/accum_run.cpp). Every form -- aligned runs, a tested uniform warp,
sorted runs, their compensated twins and the block fold -- must deliver the
exact slot sums with exactly the commits it promises, and commit lane by lane
where its vote fails or the warp is partial.

CPU: the host path (one open run per form, Neumaier in lane order) under the
address and undefined-behaviour sanitizers, and the device code compiled for
sm_103a. GPU: the kernels."""

import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
SRC = os.path.join(REPO, "tests", "cpp", "accum_run.cpp")


def _run(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "accum run ok" in r.stdout, r.stdout + r.stderr


def test_host_path(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    probe = subprocess.run([cxx, "-fsanitize=address,undefined", "-x", "c++", "-", "-o", str(tmp_path / "p")],
                           input="int main(){}", capture_output=True, text=True)
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"] if probe.returncode == 0 else []
    exe = str(tmp_path / "accum_run")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-g", "-Wall", "-Wextra", "-I", INCLUDE, SRC, "-o", exe] + san,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _run(exe)


def _nvcc(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "accum_run_cu")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "-I", INCLUDE, SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_compiles_for_sm103a(tmp_path):
    _nvcc(tmp_path)


@pytest.mark.gpu
def test_device_runs(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _run(_nvcc(tmp_path))
