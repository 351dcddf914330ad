"""ctypes binding of oracle/liboracle.so -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs, as the checker or the timed CPU baseline; never by the
aether_gb300 package. `build()` compiles the library from oracle/Makefile.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "aether_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB_PATH


class OrcOperand(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("pitch", ctypes.c_uint64)]


class OrcArgs(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint64), ("sample_offset", ctypes.c_uint32),
        ("dst", ctypes.c_void_p), ("dst_pitch", ctypes.c_uint64),
        ("operands", ctypes.POINTER(OrcOperand)), ("n_operands", ctypes.c_uint32),
        ("scalars", ctypes.POINTER(ctypes.c_double)), ("n_scalars", ctypes.c_uint32),
        ("keys", ctypes.POINTER(ctypes.c_uint64)), ("n_keys", ctypes.c_uint32),
        ("reduce_out", ctypes.POINTER(ctypes.c_double)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u64, u32, d, f, i = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_double, ctypes.c_float, ctypes.c_int
        P = ctypes.c_void_p
        sig = {
            "orc_splitmix64": (u64, [u64]),
            "orc_generator_key": (u64, [u64, u64]),
            "orc_substream_key": (u64, [u64, u64]),
            "orc_random_bits64": (u64, [u64, u32, u64]),
            "orc_uniform01_f64": (d, [u64, u32, u64]),
            "orc_uniform01_f32": (f, [u64, u32, u64]),
            "orc_normal_f64": (d, [u64, u32, u64]),
            "orc_normal_f32": (f, [u64, u32, u64]),
            "orc_eval": (i, [ctypes.c_char_p, i, ctypes.POINTER(OrcArgs), i]),
            "orc_last_error": (ctypes.c_char_p, []),
            "orc_pair_combine_f64": (None, [d, d, d, d, P, P]),
            "orc_reduce32_f64": (None, [P, P, P, P]),
            "orc_reduce32_f32": (None, [P, P, P, P]),
            "orc_fill_uniform_f64": (None, [u64, d, d, i, u64, u64, P, i]),
            "orc_fill_uniform_f32": (None, [u64, f, f, i, u64, u64, P, i]),
            "orc_fill_normal_f64": (None, [u64, d, d, i, u64, u64, P, u32, i]),
            "orc_cfg1_f64": (None, [P, P, P, P, u64, u64, i]),
            "orc_cfg2a_f64": (None, [P, P, P, P, P, u64, u64, i]),
            "orc_max_threads": (i, []),
            "orc_philox_block": (None, [u64, u32, u64, P]),
            "orc_u01_from_word_f64": (d, [u32]),
            "orc_u01_from_word_f32": (f, [u32]),
            "orc_u01_hq": (d, [u32, u32]),
            "orc_lag_fourth_moment": (None, [u64, u64, i, i, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def philox_block(seed, global_, counter):
    """The four words of the keyed Philox block of (seed, global, counter)."""
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox_block(seed, global_, counter, _ptr(out))
    return out


def lag_fourth_moment(salt, lag, n, f32=False):
    """(mean, standard error) of z^2 z'^2 over n seeds, z' `lag` counters on."""
    m, se = ctypes.c_double(), ctypes.c_double()
    lib().orc_lag_fourth_moment(salt, lag, n, int(f32), ctypes.byref(m), ctypes.byref(se))
    return m.value, se.value


def generator_key(seed, stream_id=0):
    return lib().orc_generator_key(seed, stream_id)


def substream_key(key, k):
    return lib().orc_substream_key(key, k)


def eval_ir(ir, n, operands=(), scalars=(), keys=(), out=None, mode=0, dst_comps=1, dst_dtype=np.float64,
            sample_offset=0, nthreads=0, reduce=False):
    """Evaluate an aether-ir/1 plan on host arrays.

    operands: sequence of 2-D numpy arrays (comps, pitch) holding planes.
    Returns (out, reduce_pair)."""
    L = lib()
    if out is None:
        out = np.zeros((dst_comps, max(n, 1)), dtype=dst_dtype)
    ops = (OrcOperand * max(len(operands), 1))()
    keep = []
    for k, a in enumerate(operands):
        a = np.ascontiguousarray(a)
        keep.append(a)
        ops[k].ptr = a.ctypes.data
        ops[k].pitch = a.shape[1] if a.ndim == 2 else a.shape[0]
    sc = np.asarray(scalars, dtype=np.float64)
    ky = np.asarray(keys, dtype=np.uint64)
    red = np.zeros(2, dtype=np.float64)
    args = OrcArgs()
    args.n = n
    args.sample_offset = sample_offset
    args.dst = out.ctypes.data
    args.dst_pitch = out.shape[1] if out.ndim == 2 else out.shape[0]
    args.operands = ops
    args.n_operands = len(operands)
    args.scalars = sc.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    args.n_scalars = len(sc)
    args.keys = ky.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    args.n_keys = len(ky)
    args.reduce_out = red.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    rc = L.orc_eval(ir.encode(), mode, ctypes.byref(args), nthreads)
    if rc != 0:
        raise RuntimeError("oracle: " + L.orc_last_error().decode())
    return out, (red if reduce else None)


def fill_uniform_f64(key, lo, hi, comps, n, pitch=None, nthreads=0):
    pitch = pitch or n
    out = np.zeros((comps, pitch), dtype=np.float64)
    lib().orc_fill_uniform_f64(key, lo, hi, comps, n, pitch, _ptr(out), nthreads)
    return out


def fill_uniform_f32(key, lo, hi, comps, n, pitch=None, nthreads=0):
    pitch = pitch or n
    out = np.zeros((comps, pitch), dtype=np.float32)
    lib().orc_fill_uniform_f32(key, lo, hi, comps, n, pitch, _ptr(out), nthreads)
    return out


def fill_normal_f64(key, mean, sd, comps, n, pitch=None, sample_offset=0, nthreads=0, out=None):
    pitch = pitch or n
    if out is None:
        out = np.zeros((comps, pitch), dtype=np.float64)
    assert out.dtype == np.float64 and out.flags.c_contiguous and out.shape == (comps, pitch)
    lib().orc_fill_normal_f64(key, mean, sd, comps, n, pitch, _ptr(out), sample_offset, nthreads)
    return out


def cfg1(a, b, c, nthreads=0, out=None):
    n = a.shape[1]
    d = np.zeros_like(a) if out is None else out
    assert d.shape == a.shape and d.dtype == np.float64 and d.flags.c_contiguous
    lib().orc_cfg1_f64(_ptr(a), _ptr(b), _ptr(c), _ptr(d), n, n, nthreads)
    return d


def cfg2a(a, b, c, d0, nthreads=0, out=None):
    n = a.shape[1]
    d = np.zeros_like(a) if out is None else out
    assert d.shape == a.shape and d.dtype == np.float64 and d.flags.c_contiguous
    lib().orc_cfg2a_f64(_ptr(a), _ptr(b), _ptr(c), _ptr(d0), _ptr(d), n, n, nthreads)
    return d


def max_threads():
    return lib().orc_max_threads()


# ---------------------------------------------------------------------------
# Runtime-typed strided evaluation (eval/Runtime.h:103-137 evalElement and
# :221 the scalar cast): numpy restatement over logical-shape views. numpy
# rounds every float32/float64 add and multiply on its own, as the reference's
# host loop does under -ffp-contract=off.
# ---------------------------------------------------------------------------
RT_ASSIGN, RT_ADD, RT_SUB, RT_SCALE, RT_ADD_SCALED, RT_SUB_SCALED = range(6)


def runtime_eval(op, a, b, out_dtype, scalar=0.0):
    """out = op(a, b, scalar) elementwise; a, b are numpy arrays of out's
    logical shape (any strides); returns a new array of that shape."""
    if op == RT_ASSIGN:
        return np.asarray(a).astype(out_dtype)
    t = np.asarray(a).dtype.type
    s = t(scalar)
    if op == RT_ADD:
        r = a + b
    elif op == RT_SUB:
        r = a - b
    elif op == RT_SCALE:
        r = s * a
    elif op == RT_ADD_SCALED:
        r = a + s * b
    else:
        r = a - s * b
    return np.asarray(r, dtype=out_dtype)
