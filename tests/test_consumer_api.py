"""The per-sample consumer API (include/aether: View, SampleIndex, Item,
expressions, aether::math, random leaves, launch helpers) used the way a
reference consumer uses it, checked against the oracle.

* CPU: tests/cpp/consumer_host_loop.cpp, the reference's host-loop pattern,
  compiled with contraction off: every result equals the oracle bit for bit
  (the host math facade is std::, as the oracle's).
* GPU: tests/cpp/consumer_kernels.cu, kernels written in the reference's
  spelling (tests/test_GraphCapture.cu:45-58 is the idiom) compiled unmodified
  by nvcc against -I include: Philox fills bit-exact, arithmetic and geometry
  bit-exact with --fmad=false, transcendental expressions within the native
  bound of aether_gb300.accuracy (also with the FP64-grade math facade,
  AETHER_GB300_FP64_GRADE), and the emulated-FP64 math facade within its
  bound.
"""

import os
import shutil
import subprocess

import numpy as np
import pytest

from aether_gb300 import accuracy as acc
from aether_gb300 import expr as E
from aether_gb300.expr import IrContext, Operand, plan_text

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(REPO, "aether_gb300", "lib")


def oracle_eval(oracle, build, arrays, n, dst_shape):
    """Evaluate the Python front end's tree for the same expression in the
    oracle: `build` gets one Operand per array (fake addresses) and returns
    the expression; `arrays` are (comps, n) numpy planes."""
    ops = [Operand(0x100000 * (k + 1), n, "f64", shape) for k, (shape, _) in enumerate(arrays)]
    e = build(*ops)
    ctx = IrContext()
    text = plan_text("f64", dst_shape, "set", e, ctx)
    by_addr = {op.ptr: a for op, (_, a) in zip(ops, arrays)}
    operands = [by_addr[o[0]] for o in ctx.operands]
    comps = int(np.prod(dst_shape)) if dst_shape else 1
    out, _ = oracle.eval_ir(text, n, operands=operands, scalars=ctx.scalars, keys=ctx.keys, dst_comps=comps)
    return out


def cfg2a_expr(a, b, c, d0):
    return E.cwiseSqrt(a * a + b * b) * E.cwiseLog1p(E.cwiseAbs(c)) + E.cwiseRsqrt(E.constant(1.0, (3,)) + d0 * d0)


def check_results(oracle, r, n, exact_arith, bound_expr):
    """r: dict name -> (comps, n) planes from a consumer run."""
    k42 = oracle.generator_key(42)
    fills = [("a", 0, -1.0, 1.0, 3), ("b", 1, -1.0, 1.0, 3), ("c", 2, -1.0, 1.0, 3), ("d0", 3, -4.0, 4.0, 3),
             ("q", 4, -1.0, 1.0, 4), ("m", 5, -1.0, 1.0, 9)]
    for name, s, lo, hi, comps in fills:
        ref = oracle.fill_uniform_f64(oracle.substream_key(k42, s), lo, hi, comps, n)
        assert np.array_equal(r[name], ref[:, :n]), name
    A, B, C, D0, Q, M = (r[k] for k in ("a", "b", "c", "d0", "q", "m"))

    cfg1 = oracle.cfg1(A, B, C)
    scale1 = np.maximum.reduce([np.abs(A), np.abs(B * C), np.abs(np.sin(A) * np.exp(-C * C))])
    cfg2a = oracle.cfg2a(A, B, C, D0)
    scale2 = np.maximum(np.abs(np.sqrt(A * A + B * B) * np.log1p(np.abs(C))), np.abs(1.0 / np.sqrt(1.0 + D0 * D0)))
    for name, ref, scale in (("d1", cfg1, scale1), ("d2", cfg2a, scale2)):
        if bound_expr == 0:
            assert np.array_equal(r[name], ref), name
        elif bound_expr == "native":
            e = acc.term_scale_error_ulp(r[name], ref, scale)
            assert e <= acc.NATIVE_EXPR_ULPS, (name, e)
        else:
            e = acc.term_scale_error_2m53(r[name], ref, scale)
            assert e <= bound_expr, (name, e)

    cross = oracle_eval(oracle, lambda a, b: a.cross(b), [((3,), A), ((3,), B)], n, (3,))
    qrot = oracle_eval(oracle, lambda q, b: q.quatRotate(b), [((4,), Q), ((3,), B)], n, (3,))
    inv = oracle_eval(oracle, lambda m: E.select(E.cwiseAbs(m.det()) > 1e-300, m.inverse(), E.constant(0.0, (3, 3))),
                      [((3, 3), M)], n, (3, 3))
    dot = oracle_eval(oracle, lambda a, b: a.dot(b), [((3,), A), ((3,), B)], n, ())
    for name, ref in (("cr", cross), ("qr", qrot), ("mi", inv), ("dt", dot)):
        got = r[name]
        if exact_arith:
            assert np.array_equal(got, ref[:, :n] if ref.ndim == 2 else ref), name
        else:
            # FMA contraction on the device: a few ulp of the operand products
            scale = np.maximum(np.abs(ref), 1e-300)
            assert np.max(np.abs(got - ref) / scale) < 1e-9, name


def test_host_loop_consumer_is_bit_exact(tmp_path, oracle):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "consumer_host_loop")
    src = os.path.join(REPO, "tests", "cpp", "consumer_host_loop.cpp")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-I", INCLUDE, src, "-o", exe,
                        "-L", LIBDIR, "-laether_gb300", "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n = 1037
    out = tmp_path / "host.bin"
    run = subprocess.run([exe, str(out), str(n)], capture_output=True, text=True)
    assert run.returncode == 0 and "host loop ok" in run.stdout, run.stdout + run.stderr
    raw = np.fromfile(str(out), dtype=np.float64)
    res, off = {}, 0
    for name, comps in (("a", 3), ("b", 3), ("c", 3), ("d0", 3), ("q", 4), ("m", 9), ("z", 1), ("n2", 2), ("d1", 3),
                        ("d2", 3), ("cr", 3), ("qr", 3), ("mi", 9), ("dt", 1)):
        res[name] = raw[off:off + comps * n].reshape(comps, n)
        off += comps * n
    assert off == raw.size
    check_results(oracle, res, n, exact_arith=True, bound_expr=0)
    k42 = oracle.generator_key(42)
    assert np.array_equal(res["z"], oracle.fill_normal_f64(oracle.substream_key(k42, 6), 0.0, 1.0, 1, n))
    assert np.array_equal(res["n2"], oracle.fill_normal_f64(oracle.substream_key(k42, 7), 0.5, 2.0, 2, n))


def _nvcc_build(tmp_path, name, extra):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / name)
    src = os.path.join(REPO, "tests", "cpp", "consumer_kernels.cu")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2", "-I", INCLUDE, src, "-o", exe,
           "-L", LIBDIR, "-laether_gb300", "-Xlinker", "-rpath," + LIBDIR] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_consumer_kernels_compile_for_sm103a(tmp_path):
    """Compiling needs no GPU: the reference-spelled kernels build with nvcc
    against include/ alone, in every lowering of the math facade."""
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("no nvcc")
    from aether_gb300 import _abi
    _abi.lib()
    _nvcc_build(tmp_path, "ck_default", [])
    _nvcc_build(tmp_path, "ck_exact", ["--fmad=false"])
    _nvcc_build(tmp_path, "ck_emulated", ["-DAETHER_GB300_EMULATED_FP64"])
    _nvcc_build(tmp_path, "ck_fp64_grade", ["-DAETHER_GB300_FP64_GRADE"])


def _run_kernels(tmp_path, exe, n):
    out = tmp_path / (os.path.basename(exe) + ".bin")
    run = subprocess.run([exe, str(out), str(n)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0 and "consumer kernels ok" in run.stdout, run.stdout + run.stderr
    cap = (n + 31) // 32 * 32
    raw = np.fromfile(str(out), dtype=np.float64)
    res, off = {}, 0
    for name, comps in (("a", 3), ("b", 3), ("c", 3), ("d0", 3), ("q", 4), ("m", 9), ("d1", 3), ("d2", 3), ("cr", 3),
                        ("cr2", 3), ("qr", 3), ("mi", 9), ("dt", 1)):
        res[name] = np.ascontiguousarray(raw[off:off + comps * cap].reshape(comps, cap)[:, :n])
        off += comps * cap
    assert off == raw.size
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["default", "exact", "emulated", "fp64_grade"])
def test_consumer_kernels_on_device(tmp_path, oracle, variant):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    extra = {"default": [], "exact": ["--fmad=false"], "emulated": ["-DAETHER_GB300_EMULATED_FP64"],
             "fp64_grade": ["-DAETHER_GB300_FP64_GRADE"]}[variant]
    exe = _nvcc_build(tmp_path, "ck_" + variant, extra)
    n = 4099
    res = _run_kernels(tmp_path, exe, n)
    assert np.array_equal(res["cr"], res["cr2"])
    bound = "native" if variant != "emulated" else acc.EMU_EXPR_BOUND_2M53
    check_results(oracle, res, n, exact_arith=(variant == "exact"), bound_expr=bound)


@pytest.mark.gpu
def test_array_growth_surface(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cxx = shutil.which("g++") or shutil.which("c++")
    exe = str(tmp_path / "consumer_array")
    src = os.path.join(REPO, "tests", "cpp", "consumer_array.cpp")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I", INCLUDE, src, "-o", exe, "-L", LIBDIR,
                        "-laether_gb300", "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0 and "array ok" in run.stdout, run.stdout + run.stderr
