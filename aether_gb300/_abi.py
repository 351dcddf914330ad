"""ctypes binding of include/aether_gb300.h (libaether_gb300.so).

The library is built in-tree by aether_gb300/build.py. Loading fails loudly if
it is missing: there is no other implementation of the engine to fall back on.
"""

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB


class AetherOperand(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("pitch", ctypes.c_uint64)]


class AetherLaunch(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint64), ("sample_offset", ctypes.c_uint32), ("flags", ctypes.c_uint32),
        ("dst", ctypes.c_void_p), ("dst_pitch", ctypes.c_uint64),
        ("operands", ctypes.POINTER(AetherOperand)), ("n_operands", ctypes.c_uint32),
        ("scalars", ctypes.POINTER(ctypes.c_double)), ("n_scalars", ctypes.c_uint32),
        ("keys", ctypes.POINTER(ctypes.c_uint64)), ("n_keys", ctypes.c_uint32),
        ("reduce_out", ctypes.c_void_p),
        ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_uint64),
    ]


class AetherLowering(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int), ("ipt", ctypes.c_int), ("vec", ctypes.c_int),
                ("contract", ctypes.c_int), ("math", ctypes.c_int), ("min_blocks", ctypes.c_int)]


class AetherPlanInfo(ctypes.Structure):
    _fields_ = [("hash", ctypes.c_uint64), ("n_operands", ctypes.c_int), ("n_scalars", ctypes.c_int),
                ("n_keys", ctypes.c_int), ("dst_comps", ctypes.c_int), ("dst_dtype", ctypes.c_int),
                ("is_sum", ctypes.c_int), ("block", ctypes.c_int), ("ipt", ctypes.c_int), ("vec", ctypes.c_int),
                ("registers", ctypes.c_int), ("blocks_per_sm", ctypes.c_int), ("compile_ms", ctypes.c_double)]


class AetherBatchItem(ctypes.Structure):
    _fields_ = [("plan", ctypes.c_int), ("reserved", ctypes.c_int), ("args", AetherLaunch)]


class AetherBatchInfo(ctypes.Structure):
    _fields_ = [("hash", ctypes.c_uint64), ("n_plans", ctypes.c_int), ("n_items", ctypes.c_int),
                ("total_tiles", ctypes.c_uint64), ("block", ctypes.c_int), ("ipt", ctypes.c_int),
                ("registers", ctypes.c_int), ("blocks_per_sm", ctypes.c_int), ("compile_ms", ctypes.c_double)]


class AetherServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("mode", ctypes.c_int), ("max_inflight", ctypes.c_int),
                ("max_items", ctypes.c_int), ("block", ctypes.c_int), ("ipt", ctypes.c_int),
                ("idle_spin_us", ctypes.c_int), ("upload_engine", ctypes.c_int), ("grouping", ctypes.c_int)]


class AetherServeOperand(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("host", ctypes.c_void_p), ("pitch", ctypes.c_uint64)]


class AetherServeRequest(ctypes.Structure):
    _fields_ = [("plan", ctypes.c_int), ("flags", ctypes.c_int), ("n", ctypes.c_uint64),
                ("operands", ctypes.POINTER(AetherServeOperand)), ("n_operands", ctypes.c_uint32),
                ("n_scalars", ctypes.c_uint32), ("scalars", ctypes.POINTER(ctypes.c_double)),
                ("keys", ctypes.POINTER(ctypes.c_uint64)), ("n_keys", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("host_out", ctypes.c_void_p), ("arrival_ns", ctypes.c_uint64)]


class AetherServeStatus(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("launch_items", ctypes.c_int), ("t_arrival_ns", ctypes.c_uint64),
                ("t_dispatch_ns", ctypes.c_uint64), ("t_done_ns", ctypes.c_uint64), ("output", ctypes.c_void_p),
                ("out_pitch", ctypes.c_uint64), ("bytes", ctypes.c_uint64), ("uploaded_bytes", ctypes.c_uint64)]


class AetherServeStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint64) for name in (
        "submitted", "completed", "failed", "launches", "launched_items", "bytes", "uploaded_bytes",
        "resident_hits", "resident_misses", "evictions", "arena_bytes", "arena_peak_bytes", "resident_bytes",
        "first_arrival_ns", "last_done_ns", "enqueue_ns", "admit_ns")]


class AetherRuntimeView(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype_code", ctypes.c_uint8), ("dtype_bits", ctypes.c_uint8),
                ("dtype_lanes", ctypes.c_uint16), ("rank", ctypes.c_int32),
                ("extents", ctypes.c_int64 * 6), ("strides", ctypes.c_int64 * 6)]


# name -> (restype, argtypes); every symbol include/aether_gb300.h declares.
_P = ctypes.c_void_p
_SIGS = {
    "aether_probe": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "aether_runtime_version": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "aether_last_error": (ctypes.c_char_p, []),
    "aether_chunk_alloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_size_t, _P,
                                          ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "aether_chunk_release": (None, [_P]),
    "aether_drain": (None, []),
    "aether_fill": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P]),
    "aether_copy": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _P, ctypes.c_int, ctypes.c_int, _P,
                                   ctypes.c_size_t, _P]),
    "aether_stream_wait": (ctypes.c_int, [ctypes.c_int, _P, _P]),
    "aether_stream_sync": (ctypes.c_int, [ctypes.c_int, _P]),
    "aether_stream_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
    "aether_current_device": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "aether_pointer_device": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    "aether_memory_v1": (_P, []),
    "aether_gb300_v1": (_P, []),
    "aether_stream_destroy": (None, [_P]),
    "aether_plan_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(AetherLowering), ctypes.POINTER(_P)]),
    "aether_plan_info": (ctypes.c_int, [_P, ctypes.POINTER(AetherPlanInfo)]),
    "aether_plan_workspace_size": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    "aether_plan_launch": (ctypes.c_int, [_P, ctypes.POINTER(AetherLaunch), _P]),
    "aether_plan_source": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "aether_plan_release": (None, [_P]),
    "aether_plan_launch_noalloc": (ctypes.c_int, [_P, ctypes.POINTER(AetherLaunch), _P]),
    "aether_batch_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.POINTER(AetherLowering),
                                           ctypes.POINTER(_P)]),
    "aether_batch_set_items": (ctypes.c_int, [_P, ctypes.POINTER(AetherBatchItem), ctypes.c_int, _P]),
    "aether_batch_launch": (ctypes.c_int, [_P, _P]),
    "aether_batch_capture": (ctypes.c_int, [_P, _P]),
    "aether_batch_replay": (ctypes.c_int, [_P, _P]),
    "aether_batch_info": (ctypes.c_int, [_P, ctypes.POINTER(AetherBatchInfo)]),
    "aether_batch_release": (None, [_P]),
    "aether_plan_launch_many": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(AetherLaunch), ctypes.c_int, _P]),
    "aether_serve_open": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.POINTER(AetherServeConfig),
                                         ctypes.POINTER(_P)]),
    "aether_serve_submit": (ctypes.c_int, [_P, ctypes.POINTER(AetherServeRequest), ctypes.POINTER(ctypes.c_uint64)]),
    "aether_serve_feed": (ctypes.c_int, [_P, ctypes.POINTER(AetherServeRequest), ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_uint64)]),
    "aether_serve_status": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.POINTER(AetherServeStatus)]),
    "aether_serve_wait": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(AetherServeStatus)]),
    "aether_serve_release": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "aether_serve_stats": (ctypes.c_int, [_P, ctypes.POINTER(AetherServeStats)]),
    "aether_serve_close": (None, [_P]),
    "aether_runtime_eval": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(AetherRuntimeView),
                                           ctypes.POINTER(AetherRuntimeView), ctypes.POINTER(AetherRuntimeView),
                                           ctypes.c_double, _P]),
    "aether_plan_generate": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(AetherLowering), ctypes.c_char_p,
                                            ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "aether_nvrtc_check": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p]),
    "aether_rtc_header_count": (ctypes.c_int, []),
    "aether_rtc_header": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                         ctypes.POINTER(ctypes.c_char_p)]),
    "aether_rtc_digest": (ctypes.c_uint64, []),
    "aether_plan_cache_key": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                             ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64)]),
    "aether_rtc_compile": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p),
                                          ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_size_t)]),
}

_lib = None


class AetherError(RuntimeError):
    pass


def lib():
    """Load libaether_gb300.so (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.environ.get("AETHER_GB300_REBUILD"):
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise AetherError("libaether_gb300.so is missing; run python -m aether_gb300.build")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != 0:
        msg = lib().aether_last_error()
        raise AetherError((msg or b"").decode(errors="replace") or "aether call failed (status %d)" % rc)
    return rc


def lowering(block=0, ipt=0, vec=0, contract=-1, math=0, min_blocks=0):
    return AetherLowering(block, ipt, vec, contract, math, min_blocks)


def generate(ir, low=None):
    L = lib()
    n = ctypes.c_size_t(0)
    check(L.aether_plan_generate(ir.encode(), ctypes.byref(low) if low else None, None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    check(L.aether_plan_generate(ir.encode(), ctypes.byref(low) if low else None, buf, n.value + 1, ctypes.byref(n)))
    return buf.value.decode()


def nvrtc_check(source, arch="sm_103a"):
    check(lib().aether_nvrtc_check(source.encode(), arch.encode()))
