"""The C-ABI library without a GPU: it loads, exports every symbol that
include/*.h declares, and its offline lowering checks and compiles plans
(NVRTC cross-compiles for sm_103a without a device)."""

import ctypes
import glob
import os
import re

import pytest

from conftest import REPO


def _declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(aether_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_loads_and_exports_every_declared_symbol():
    from aether_gb300 import _abi
    L = _abi.lib()
    declared = _declared_symbols()
    assert len(declared) >= 15
    for name in sorted(declared):
        assert hasattr(L, name), "libaether_gb300.so does not export " + name
    # The Python binding covers every declared symbol too.
    assert declared <= set(_abi._SIGS), declared - set(_abi._SIGS)


def test_only_aether_symbols_are_exported():
    import subprocess
    from aether_gb300 import _abi
    _abi.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", _abi.LIB_PATH], capture_output=True, text=True).stdout
    funcs = [l.split()[-1] for l in out.splitlines() if " T " in l]
    assert funcs and all(f.startswith("aether_") for f in funcs), funcs


def test_probe_without_device_fails_cleanly():
    import torch
    from aether_gb300 import _abi
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    n = ctypes.c_int(0)
    assert _abi.lib().aether_probe(ctypes.byref(n)) == 1
    assert _abi.lib().aether_last_error()


import aether_gb300 as ag
from aether_gb300 import _abi
from aether_gb300.expr import IrContext, Operand, plan_text


def _leaf(k, shape=(3,), dt="f64"):
    return Operand(0x10000 * (k + 1), 1024, dt, shape)


def _corpus():
    a, b, c, d0 = (_leaf(k) for k in range(4))
    q, p = _leaf(4, (4,)), _leaf(5, (4,))
    M = _leaf(6, (3, 3))
    x, y = _leaf(7, (8,), "f32"), _leaf(8, (8,), "f32")
    g = ag.Generator(7)
    yield "cfg1", "f64", (3,), "set", a + b * c + ag.cwiseSin(a) * ag.cwiseExp((c * c) * (-1.0))
    yield "cfg2a", "f64", (3,), "set", (ag.cwiseSqrt(a * a + b * b) * ag.cwiseLog1p(ag.cwiseAbs(c))
                                       + ag.cwiseRsqrt(ag.constant(1.0, (3,)) + d0 * d0))
    yield "normal", "f64", (1,), "set", g.substream(4).normal(1, 0.0, 1.0)
    yield "uniform", "f64", (3,), "set", g.substream(0).uniform(3, -4.0, 4.0)
    yield "cross", "f64", (3,), "set", a.cross(b)
    yield "qrot", "f64", (3,), "set", q.quatRotate(a)
    yield "qmul", "f64", (4,), "set", q.quatMul(p)
    yield "inv_guard", "f64", (3, 3), "set", ag.select(ag.cwiseAbs(M.det()) > 1e-300, M.inverse(),
                                                       ag.constant(0.0, (3, 3)))
    yield "dot_sum_f32", "f32", (), "setsum", x.dot(y)
    yield "sum_f64", "f64", (), "sum", a.dot(b)
    yield "accumulate", "f64", (3,), "add", a * 2.0
    yield "unit_view", "f64", (3,), "set", a * a.rNorm().at_sample0()
    yield "matmul", "f64", (3, 3), "set", M.matmul(M.transpose())
    yield "lognormal_f32", "f32", (2,), "set", g.lognormal(2, 0.1, 0.5)
    yield "clamp_pow", "f64", (3,), "set", ag.clamp(ag.cwisePow(ag.cwiseAbs(a), 1.5), -2.0, 2.0)


@pytest.mark.parametrize("case", list(_corpus()), ids=lambda c: c[0])
@pytest.mark.parametrize("contract, math", [(0, 0), (1, 0), (0, 1), (0, 2), (0, 3)])
def test_corpus_lowers_and_compiles_for_sm103a(case, contract, math):
    # math 1 (double-float for f64 plans), 2 (float-float for f32/ff plans)
    # and 3 (triple-float for f64 plans) lower the same corpus through the
    # emulated generator
    name, dt, shape, op, e = case
    ir = plan_text(dt, shape, op, e, IrContext())
    src = _abi.generate(ir, _abi.lowering(contract=contract, math=math))
    assert re.search(r"ag_(expr|fill|sum)_[0-9a-f]{8}(_tf)?_v\(", src) and re.search(r"ag_(expr|fill|sum)_[0-9a-f]{8}(_tf)?_s\(", src)
    if math == 3 and dt == "f64":
        assert "_tf_v(" in src
    _abi.nvrtc_check(src, "sm_103a")


@pytest.mark.parametrize("bad, msg", [
    ("(plan f64 [3] set (add (in 0 f64 [3]) (in 1 f64 [2])))", "shapes differ"),
    ("(plan f64 [2] set (in 0 f64 [3]))", "does not match"),
    ("(plan f64 [3] set (frob (in 0 f64 [3])))", "unknown node"),
    ("(plan f64 [3] set (in 0 f64 [3])", "unexpected end"),
    ("(plan f64 [3] set (cross (in 0 f64 [4]) (in 1 f64 [4])))", "cross"),
    ("(plan f64 [] sum (in 0 f64 [3]))", "does not match"),
    ("(plan f64 [3] set (in 1 f64 [3]))", "unused"),
    ("(plan f64 [3] set (select (in 0 f64 [3]) (in 0 f64 [3]) (in 0 f64 [3])))", "boolean"),
    ("(plan q64 [3] set (in 0 f64 [3]))", "dtype"),
])
def test_bad_plans_are_rejected_with_a_message(bad, msg):
    with pytest.raises(ag.AetherError, match=msg):
        _abi.generate(bad)


def test_structural_cse_shares_subtrees():
    a = _leaf(0)
    e = ag.cwiseSin(a) * ag.cwiseSin(a)
    src = _abi.generate(plan_text("f64", (3,), "set", e, IrContext()))
    assert src.count("ag::f_sin(") == 3   # once per component, not twice


def _fast_path(src):
    """The double-float lane loop of a generated source (without the native
    recomputation function)."""
    return src[src.index("ag_chunk"):]


def test_emulated_products_are_range_checked_only_where_bounds_need_it():
    # inputs of the double-float path lie in [2^-50, 2^60]: a*a + b*b, the
    # square root and log1p of |c| keep every product above 2^-102, so the
    # config-2a tree carries no product check; a product of three inputs
    # can reach 2^-150 and is checked; exp carries its own range flag
    a, b, c, d0 = (_leaf(k) for k in range(4))
    cfg2a = (ag.cwiseSqrt(a * a + b * b) * ag.cwiseLog1p(ag.cwiseAbs(c))
             + ag.cwiseRsqrt(ag.constant(1.0, (3,)) + d0 * d0))
    src = _fast_path(_abi.generate(plan_text("f64", (3,), "set", cfg2a, IrContext()), _abi.lowering(math=1)))
    assert "ag::e64::ck(" not in src
    assert src.count("ag::e64::from_double_ck(") == 12
    # constant(1.0) is baked in, so the bounds also keep the output in range
    assert "(lit 0x1.0000000000000p+0)" in plan_text("f64", (3,), "set", cfg2a, IrContext())
    assert "out_ok(" not in src
    src = _fast_path(_abi.generate(plan_text("f64", (3,), "set", (a * b) * c, IrContext()), _abi.lowering(math=1)))
    assert src.count("ag::e64::ck(") == 3          # the outer product, once per component
    src = _fast_path(_abi.generate(plan_text("f64", (3,), "set", ag.cwiseExp(a) * b, IrContext()),
                                   _abi.lowering(math=1)))
    assert src.count("ag::e64::exp_(") == 3 and src.count(", ok_)") >= 6
    # exact f32 operands are not range checked, so their products are
    x, y = _leaf(7, (8,), "f32"), _leaf(8, (8,), "f32")
    src = _fast_path(_abi.generate(plan_text("f32", (8,), "set", x * y, IrContext()), _abi.lowering(math=2)))
    assert src.count("ag::e64::ck(ag::e64::two_prod(") == 8


def test_emulated_math_requires_f64_plan():
    a = _leaf(0, (3,), "f32")
    ir = plan_text("f32", (3,), "set", a + a, IrContext())
    src = _abi.generate(ir, _abi.lowering(math=1))
    assert "ag_emu64" in src


def test_seam_table_matches_the_reference_layout():
    """aether_memory_v1 returns the dsc/src/seam.h:22-53 table (ABI 2) whose
    entries are this library's own functions; FFT answers optional-missing."""
    import ctypes
    from aether_gb300 import _abi
    L = _abi.lib()
    P = ctypes.c_void_p
    names = ["probe", "runtime_version", "current_device", "last_error", "chunk_alloc", "chunk_release", "drain",
             "fill", "copy", "stream_wait", "stream_sync", "pointer_device", "fft_plan", "fft_exec", "fft_destroy"]

    class Mem(ctypes.Structure):
        _fields_ = [("abi", ctypes.c_uint32)] + [(n, P) for n in names]

    t = ctypes.cast(L.aether_memory_v1(), ctypes.POINTER(Mem)).contents
    assert t.abi == 2
    for n in names[:12]:
        assert t.__getattribute__(n) == ctypes.cast(getattr(L, "aether_" + n), P).value, n
    fft_plan = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, P, ctypes.c_int, P, P, ctypes.POINTER(P))(t.fft_plan)
    plan = P(1)
    assert fft_plan(0, 0, 1, 0, 1, 1, None, 1, None, None, ctypes.byref(plan)) == 2
    assert plan.value is None and b"FFT" in L.aether_last_error()


def test_gb300_table_binds_every_path_entry():
    import ctypes
    from aether_gb300 import _abi
    L = _abi.lib()
    P = ctypes.c_void_p
    names = ["stream_create", "stream_destroy", "plan_create", "plan_info", "plan_workspace_size", "plan_launch",
             "plan_source", "plan_release", "plan_launch_noalloc", "plan_launch_many", "batch_create",
             "batch_set_items", "batch_launch", "batch_capture", "batch_replay", "batch_info", "batch_release",
             "serve_open", "serve_submit", "serve_feed", "serve_status", "serve_wait", "serve_release", "serve_stats",
             "serve_close", "runtime_eval", "rtc_header_count", "rtc_header", "rtc_digest", "plan_generate",
             "nvrtc_check", "plan_cache_key", "rtc_compile"]

    class T(ctypes.Structure):
        _fields_ = [("abi", ctypes.c_uint32), ("memory", P)] + [(n, P) for n in names]

    t = ctypes.cast(L.aether_gb300_v1(), ctypes.POINTER(T)).contents
    assert t.abi == 1 and t.memory == L.aether_memory_v1()
    for n in names:
        assert getattr(t, n) == ctypes.cast(getattr(L, "aether_" + n), P).value, n


def test_cache_key_covers_every_payload_header():
    # A kernel cached on disk must never be served after any header it may
    # include changes: flipping one byte of any payload header (the
    # Box-Muller headers included) gives a new key.
    from aether_gb300 import _abi
    L = _abi.lib()

    def key(idx=-1, src=None):
        k = ctypes.c_uint64()
        _abi.check(L.aether_plan_cache_key(b"extern \"C\" __global__ void k() {}", b"sm_103a", b"plan", idx, src,
                                           ctypes.byref(k)))
        return k.value

    base = key()
    assert key() == base
    n = L.aether_rtc_header_count()
    assert n >= 5
    seen = {base}
    for i in range(n):
        name = ctypes.c_char_p()
        text = ctypes.c_char_p()
        _abi.check(L.aether_rtc_header(i, ctypes.byref(name), ctypes.byref(text)))
        assert key(i, text.value) == base, name.value     # the same text: the same key
        edited = bytearray(text.value)
        edited[len(edited) // 2] ^= 1
        k = key(i, bytes(edited))
        assert k not in seen, name.value
        seen.add(k)
    assert L.aether_plan_cache_key(b"x", b"sm_103a", b"plan", n, b"", ctypes.byref(ctypes.c_uint64())) == 1


def test_plugin_library_exports_exactly_the_seam_table():
    # libaether_cuda.so is the drop-in for the reference's CUDA plugin: one
    # exported symbol, aether_memory_v1, as dsc/src/plugin.map declares
    import subprocess
    from aether_gb300 import _abi, build
    _abi.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", build.PLUGIN], capture_output=True, text=True).stdout
    funcs = sorted(l.split()[-1] for l in out.splitlines() if l.split() and l.split()[-2] in ("T", "D", "R", "B"))
    assert funcs == ["aether_memory_v1"], funcs
    P = ctypes.CDLL(build.PLUGIN)
    P.aether_memory_v1.restype = ctypes.c_void_p
    abi = ctypes.cast(P.aether_memory_v1(), ctypes.POINTER(ctypes.c_uint32)).contents.value
    assert abi == 2
