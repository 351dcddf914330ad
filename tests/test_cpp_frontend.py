"""The C++ front end (include/aether): a consumer program compiles against the
headers alone with a host C++ compiler, and every assignment it builds has
exactly the aether-ir/1 text the Python front end writes for the same tree,
with the same operand, scalar and key slots."""

import os
import shutil
import subprocess

import pytest

from aether_gb300 import expr as E
from aether_gb300.expr import Generator, IrContext, Operand, plan_text

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(src, out, link=False):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(REPO, "include"), src, "-o", out]
    if link:
        lib = os.path.join(REPO, "aether_gb300", "lib")
        cmd += ["-L", lib, "-laether_gb300", "-Wl,-rpath," + lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _python_texts():
    n = 1000
    a, b, c, d0 = (Operand(0x10000 * (k + 1), n, "f64", (3,)) for k in range(4))
    out = {}

    def emit(name, dtype, shape, e, op="set"):
        ctx = IrContext()
        out[name] = (plan_text(dtype, shape, op, e, ctx), len(ctx.operands), len(ctx.scalars), len(ctx.keys))

    emit("cfg1", "f64", (3,), a + b * c + E.cwiseSin(a) * E.cwiseExp((c * c) * (-1.0)))
    emit("cfg2a", "f64", (3,), E.cwiseSqrt(a * a + b * b) * E.cwiseLog1p(E.cwiseAbs(c)) +
         E.cwiseRsqrt(E.constant(1.0, (3,)) + d0 * d0))
    emit("uniform", "f64", (3,), Generator(42).substream(0).uniform(3, -1.0, 1.0))
    emit("normal", "f64", (1,), Generator(7).substream(4).normal(1, 0.0, 1.0))
    m3 = E.stack(*(E.Scalar(v) for v in (-1.0, 0.0, 2.5)))
    s3 = E.stack(*(E.Scalar(v) for v in (0.5, 1.0, 3.0)))
    l3 = E.stack(*(E.Scalar(v) for v in (0.5, 2.0, 8.0)))
    emit("normal_item", "f64", (3,), Generator(21).substream(0).normal(3, m3, s3))
    emit("exponential_item", "f64", (3,), Generator(21).substream(2).exponential(3, l3))
    q = Operand(0x70000, n, "f64", (4,))
    m = Operand(0x80000, n, "f64", (3, 3))
    emit("cross", "f64", (3,), a.cross(b))
    emit("qrot", "f64", (3,), q.quatRotate(b))
    emit("inv", "f64", (3, 3), E.select(E.cwiseAbs(m.det()) > 1e-300, m.inverse(), E.constant(0.0, (3, 3))))
    x, y = Operand(0xA0000, n, "f32", (8,)), Operand(0xB0000, n, "f32", (8,))
    emit("dot8", "f32", (), x.dot(y))
    emit("axpy_add", "f64", (3,), a * 2.5 + b / 4.0, op="add")
    emit("minmax", "f64", (3,), E.cwiseMax(E.cwiseMin(a, b), -0.5) - E.clamp(c, -0.25, 0.25))
    emit("structural", "f64", (3,), m.row(1) + m.col(2) + m.transpose().matvec(a))
    emit("literal", "f64", (3,), a * E.literal(0.1) + E.literal(-3.0))
    return out


def test_cpp_front_end_writes_the_python_ir(tmp_path):
    exe = _compile(os.path.join(REPO, "tests", "cpp", "consumer_ir.cpp"), str(tmp_path / "consumer_ir"))
    r = subprocess.run([exe], capture_output=True, text=True, check=True)
    got = {}
    for line in r.stdout.splitlines():
        name, text, nops, nsc, nkeys = line.split("\t")
        got[name] = (text, int(nops), int(nsc), int(nkeys))
    want = _python_texts()
    assert set(got) == set(want)
    for name in want:
        assert got[name] == want[name], name


def test_cpp_generator_keys_match():
    # splitmix64 keying of random/Generator.h:64-81 on both sides
    g = Generator(42)
    assert g.substream(0).key != g.substream(1).key
    assert Generator(7, 3).key == E.splitmix64(7 ^ E.splitmix64(3))


@pytest.mark.gpu
def test_cpp_consumer_on_device(tmp_path, oracle):
    """The config-1 program through the C++ headers equals the Python front
    end bit for bit (same plans), and its uniforms equal the oracle's."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import numpy as np
    import aether_gb300 as ag
    exe = _compile(os.path.join(REPO, "tests", "cpp", "consumer_cfg1.cpp"), str(tmp_path / "consumer_cfg1"), link=True)
    n = 4099
    out = tmp_path / "cfg1.bin"
    r = subprocess.run([exe, str(out), str(n)], capture_output=True, text=True)
    assert r.returncode == 0 and "consumer ok" in r.stdout, r.stdout + r.stderr
    cap = (n + 31) // 32 * 32
    raw = np.fromfile(str(out), dtype=np.float64)
    planes = raw[: 4 * 3 * cap].reshape(4, 3, cap)[:, :, :n]
    hi, comp = raw[4 * 3 * cap:]
    # Python front end, same expression and lowering
    g = ag.Generator(42)
    arrs = [ag.Array("f64", (3,), n) for _ in range(3)]
    for k, x in enumerate(arrs):
        ag.assign(x, g.substream(k).uniform(3, -1.0, 1.0))
    a, b, c = (x.view() for x in arrs)
    d = ag.Array("f64", (3,), n)
    ag.assign(d, a + b * c + ag.cwiseSin(a) * ag.cwiseExp((c * c) * (-1.0)))
    s = ag.global_sum(a.dot(b), n).cpu().numpy()
    for k, x in enumerate(arrs + [d]):
        assert np.array_equal(planes[k], x.host())
    assert hi == s[0] and comp == s[1]
    k42 = oracle.generator_key(42)
    for k in range(3):
        ref = oracle.fill_uniform_f64(oracle.substream_key(k42, k), -1.0, 1.0, 3, n)
        assert np.array_equal(planes[k], ref[:, :n])


def test_cpp_partition_algebra(tmp_path):
    exe = _compile(os.path.join(REPO, "tests", "cpp", "partition_check.cpp"), str(tmp_path / "partition_check"))
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and "partition ok" in r.stdout, r.stdout


@pytest.mark.gpu
def test_cpp_device_flag(tmp_path):
    """A consumer kernel sets DeviceFlag through DeviceFlagView; the host
    reads it (sticky), checkAndClear throws once and clears."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    lib = os.path.join(REPO, "aether_gb300", "lib")
    exe = str(tmp_path / "device_flag")
    r = subprocess.run([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I",
                        os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "device_flag.cu"),
                        "-L", lib, "-laether_gb300", "-Xlinker", "-rpath," + lib, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and "device flag ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_batch_and_server(tmp_path):
    """gb300::Batch (one launch and a graph replay) and gb300::Server through
    the C++ headers equal plain per-array assignments bit for bit."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = _compile(os.path.join(REPO, "tests", "cpp", "consumer_batch.cpp"), str(tmp_path / "consumer_batch"), link=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and "batch and serve ok" in r.stdout, r.stdout + r.stderr
