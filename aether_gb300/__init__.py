"""aether_gb300: GB300-native fused batched-expression engine.

Python host mirror of the reference's consumer surface for the fused
assignment path. Arrays are SoA (component planes at a pitch of the capacity,
a multiple of 32 samples: array/Array.h:80,288-304); expressions are built
lazily (expr.py) and `assign(dst, expr)` evaluates `dst[i] = expr` for every
sample in one sm_103a kernel generated from the tree and cached by its hash.

Device memory and streams come from PyTorch; every kernel comes from
libaether_gb300.so. There is no CPU evaluation path in this package.
"""

import ctypes
import threading

from . import _abi
from ._abi import AetherError, lowering
from .expr import (Expr, Generator, IrContext, Operand, Scalar, clamp, constant, cwiseAbs, cwiseAcos, cwiseAsin,
                   cwiseAtan, cwiseCbrt, cwiseCeil, cwiseCos, cwiseCosh, cwiseDiv, cwiseErf, cwiseExp, cwiseExp2,
                   cwiseExpm1, cwiseFloor, cwiseLog, cwiseLog10, cwiseLog1p, cwiseLog2, cwiseMax, cwiseMin, cwiseMul,
                   cwisePow, cwiseRsqrt, cwiseSign, cwiseSin, cwiseSinh, cwiseSqrt, cwiseSquare, cwiseTan, cwiseTanh,
                   cwiseTrunc, literal, plan_text, select, splitmix64, stack)

CAPACITY_ALIGNMENT = 32
_DTYPES = {"f64": 8, "f32": 4}


def quantized_capacity(n):
    """Array capacity: n rounded up to a multiple of 32 samples (array/Array.h:80, :288-295)."""
    return max(CAPACITY_ALIGNMENT, (int(n) + CAPACITY_ALIGNMENT - 1) // CAPACITY_ALIGNMENT * CAPACITY_ALIGNMENT)


def _torch():
    import torch
    return torch


def _tdtype(dtype):
    torch = _torch()
    return {"f64": torch.float64, "f32": torch.float32, "ff": torch.float32}[dtype]


class Array:
    """Owning SoA array on the GPU: `shape` components x `n` samples.

    `data` is a torch tensor (planes, capacity); plane c starts at
    c * capacity elements, 256-byte aligned for both f64 and f32. An "ff"
    array (the precision form's float-float storage) holds the hi planes of
    its components followed by their lo planes."""

    def __init__(self, dtype, shape, n, device="cuda", data=None):
        if isinstance(shape, int):
            shape = (shape,)
        self.dtype = dtype
        self.shape = tuple(shape)
        self.comps = 1
        for s in self.shape:
            self.comps *= s
        self.planes = self.comps * (2 if dtype == "ff" else 1)
        self.n = int(n)
        if data is not None:
            self.data = data
            self.capacity = data.stride(0) if data.shape[0] > 1 else max(data.stride(0), data.shape[1])
        else:
            self.capacity = quantized_capacity(n)
            self.data = _torch().zeros((self.planes, self.capacity), dtype=_tdtype(dtype), device=device)

    def host_ff(self):
        """An ff array's values, hi + lo, as float64 (comps, n)."""
        import numpy as np
        h = self.data[: self.comps, : self.n].cpu().numpy().astype(np.float64)
        lo = self.data[self.comps:, : self.n].cpu().numpy().astype(np.float64)
        return h + lo

    @classmethod
    def wrap(cls, tensor, shape=None, n=None):
        """View a (components, pitch) tensor as an array without copying."""
        dtype = {"torch.float64": "f64", "torch.float32": "f32"}[str(tensor.dtype)]
        shape = shape or (tensor.shape[0],)
        return cls(dtype, shape, n if n is not None else tensor.shape[1], data=tensor)

    @classmethod
    def from_dlpack(cls, obj, shape=None, n=None):
        """Zero-copy import of a DLPack-exporting (planes, pitch) buffer
        (interop/DLPack.h:226-430): any framework's device tensor."""
        t = _torch().utils.dlpack.from_dlpack(obj)
        if t.dim() == 1:
            t = t.reshape(1, -1)
        if t.dim() != 2 or t.stride(1) != 1:
            raise AetherError("from_dlpack: need a (planes, pitch) buffer with unit sample stride")
        return cls.wrap(t, shape=shape, n=n)

    def __dlpack__(self, stream=None):
        """DLPack export of the (planes, n) samples, plane stride = capacity."""
        v = self.data[:, : self.n]
        return v.__dlpack__() if stream is None else v.__dlpack__(stream=stream)

    def __dlpack_device__(self):
        return self.data.__dlpack_device__()

    def samples(self):
        return self.n

    def view(self):
        """The array as an expression leaf (deviceView() of the reference)."""
        return Operand(self.data.data_ptr(), self.capacity, self.dtype, self.shape, owner=self)

    __call__ = view

    def host(self):
        return self.data[:, : self.n].cpu().numpy()

    def upload(self, host):
        torch = _torch()
        t = torch.as_tensor(host).to(self.data.dtype)
        self.data[:, : self.n].copy_(t.reshape(self.comps, self.n))
        return self


class AccumPlane:
    """Per-sample compensated accumulation (accum/AccumPlane.h:43-502): a value
    plane and a compensation plane per component. `add(expr)` evaluates
    `plane += expr` in one kernel, the exact residual of each addition going
    to the compensation plane; with atomic=True the additions are atomic, so
    producers on different streams may accumulate concurrently (the
    CompensatedAtomic policy). `delivered()` is value + compensation."""

    dtype = "f64"

    def __init__(self, shape, n, device="cuda"):
        self.shape = (shape,) if isinstance(shape, int) else tuple(shape)
        self.comps = 1
        for e in self.shape:
            self.comps *= e
        self.n = int(n)
        self.capacity = quantized_capacity(n)
        self.data = _torch().zeros((2 * self.comps, self.capacity), dtype=_torch().float64, device=device)

    def add(self, expr, atomic=False, stream=None, **low):
        L = prepare(self, expr, op="accat" if atomic else "acc", **low)
        L(stream)
        return self

    def value(self):
        return Operand(self.data.data_ptr(), self.capacity, "f64", self.shape, owner=self)

    def compensation(self):
        return Operand(self.data.data_ptr() + self.comps * self.capacity * 8, self.capacity, "f64", self.shape,
                       owner=self)

    def delivered(self, stream=None):
        out = Array("f64", self.shape, self.n)
        assign(out, self.value() + self.compensation(), stream=stream)
        return out

    def zero(self):
        self.data.zero_()
        return self


class _PinnedChunk:
    """Owner of one aether_chunk_alloc pinned host chunk (released with it)."""

    def __init__(self, nbytes):
        self.chunk, self.ptr = ctypes.c_void_p(), ctypes.c_void_p()
        _abi.check(_abi.lib().aether_chunk_alloc(2, 0, nbytes, None, ctypes.byref(self.chunk), ctypes.byref(self.ptr)))

    def __del__(self):
        if self.chunk:
            _abi.lib().aether_chunk_release(self.chunk)
            self.chunk = ctypes.c_void_p()


def pinned_empty(shape, dtype="f64"):
    """Page-locked, device-mapped host memory from aether_chunk_alloc (kind 2)
    as a CPU torch tensor; the chunk is released when the last view of it
    goes away."""
    import numpy as np
    npdt = {"f64": np.float64, "f32": np.float32, "i32": np.int32, "u8": np.uint8}[dtype]
    n = 1
    for e in shape:
        n *= int(e)
    nbytes = n * np.dtype(npdt).itemsize
    owner = _PinnedChunk(max(nbytes, 1))
    buf = (ctypes.c_char * max(nbytes, 1)).from_address(owner.ptr.value)
    buf._owner = owner   # the array keeps the buffer, the buffer keeps the chunk
    return _torch().from_numpy(np.frombuffer(buf, dtype=npdt, count=n).reshape(tuple(shape)))


def padded_block_samples(n, parts, pad_to=32):
    """Block pitch of a sample-mode partition: ceil(n / parts) rounded up to
    pad_to (residency/Partition.h:61-72)."""
    if parts <= 0:
        raise AetherError("padded_block_samples failed on n/a, size=%d bytes (parts must be > 0)" % n)
    if pad_to <= 0:
        raise AetherError("padded_block_samples failed on n/a, size=%d bytes (pad_to must be > 0)" % n)
    per = (int(n) + parts - 1) // parts
    return (per + pad_to - 1) // pad_to * pad_to


def partition_view(arr, parts, r, pad_to=32):
    """Block r of `parts` of an array's sample mode (residency/Partition.h:
    104-168): starts at sample r * padded, holds min(padded, n - r * padded)
    real samples, same plane pitch, same memory."""
    if r < 0 or r >= parts:
        raise AetherError("partition_view failed on cuda:0, size=0 bytes (block index %d >= spec.parts=%d)" % (r, parts))
    padded = padded_block_samples(arr.n, parts, pad_to)
    off = r * padded
    real = max(0, min(padded, arr.n - off))
    start = min(off, arr.capacity)
    return Array.wrap(arr.data[:, start:start + real], shape=arr.shape, n=real)


class Plan:
    """A compiled plan: one aether-ir/1 text, one kernel."""

    def __init__(self, ir, low=None):
        self.ir = ir
        self.low = low
        h = ctypes.c_void_p()
        _abi.check(_abi.lib().aether_plan_create(ir.encode(), ctypes.byref(low) if low else None, ctypes.byref(h)))
        self.handle = h

    def info(self):
        i = _abi.AetherPlanInfo()
        _abi.check(_abi.lib().aether_plan_info(self.handle, ctypes.byref(i)))
        return i

    def source(self):
        n = ctypes.c_size_t()
        _abi.check(_abi.lib().aether_plan_source(self.handle, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value + 1)
        _abi.check(_abi.lib().aether_plan_source(self.handle, buf, n.value + 1, ctypes.byref(n)))
        return buf.value.decode()

    @property
    def name(self):
        """The kernel's base name (its vectorised and scalar kernels add _v / _s)."""
        import re
        m = re.search(r"\b(ag_(?:expr|fill|sum)_[0-9a-f]{8}(?:_tf)?)_v\b", self.source())
        return m.group(1) if m else None

    def workspace_size(self, n):
        b = ctypes.c_uint64()
        _abi.check(_abi.lib().aether_plan_workspace_size(self.handle, n, ctypes.byref(b)))
        return b.value

    def __del__(self):
        try:
            if self.handle:
                _abi.lib().aether_plan_release(self.handle)
        except Exception:
            pass


_cache = {}
_cache_lock = threading.Lock()


def get_plan(ir, block=0, ipt=0, vec=0, contract=-1, math=0, min_blocks=0):
    key = (ir, block, ipt, vec, contract, math, min_blocks)
    with _cache_lock:
        p = _cache.get(key)
    if p is None:
        p = Plan(ir, lowering(block, ipt, vec, contract, math, min_blocks))
        with _cache_lock:
            _cache[key] = p
    return p


class Launch:
    """A plan bound to its arguments: re-launchable without rebuilding the IR."""

    def __init__(self, plan, ctx, n, dst_ptr, dst_pitch, sample_offset=0, reduce_ptr=None, workspace=None):
        self.plan = plan
        self._ops = (_abi.AetherOperand * max(1, len(ctx.operands)))()
        for i, (ptr, pitch, _dt, _c, _owner) in enumerate(ctx.operands):
            self._ops[i].ptr = ptr
            self._ops[i].pitch = pitch
        self._owners = [o[4] for o in ctx.operands]
        self._sc = (ctypes.c_double * max(1, len(ctx.scalars)))(*ctx.scalars)
        self._keys = (ctypes.c_uint64 * max(1, len(ctx.keys)))(*ctx.keys)
        a = _abi.AetherLaunch()
        a.n = n
        a.sample_offset = sample_offset
        a.dst = dst_ptr or 0
        a.dst_pitch = dst_pitch
        a.operands = self._ops
        a.n_operands = len(ctx.operands)
        a.scalars = self._sc
        a.n_scalars = len(ctx.scalars)
        a.keys = self._keys
        a.n_keys = len(ctx.keys)
        a.reduce_out = reduce_ptr or 0
        if workspace is not None:
            a.workspace = workspace.data_ptr()
            a.workspace_bytes = workspace.numel() * workspace.element_size()
        self.args = a

    def __call__(self, stream=None):
        s = stream if stream is not None else _torch().cuda.current_stream().cuda_stream
        _abi.check(_abi.lib().aether_plan_launch(self.plan.handle, ctypes.byref(self.args), ctypes.c_void_p(s)))


def prepare(dst, expr, op="set", n=None, sample_offset=0, reduce_out=None, workspace=None, tune=False, **low):
    """Lower `dst <op>= expr` and bind its arguments; returns a Launch.

    Lowering keywords (include/aether_gb300.h AetherLowering): math = 0 FP64
    on the FP64 pipe, 1 double-float FP64 emulation (about 48 bits), 2 the
    precision form (f32/ff storage, float-float arithmetic), 3 FP64-grade
    triple-float on the FP32/INT pipes (f64 plans, the FP64 contract);
    contract (FMA contraction), block, ipt, vec, min_blocks.

    tune=True takes the autotuned lowering of this plan on this device (see
    tune.py), timing the candidates first if none is cached. Only plans that
    overwrite their destination are tuned (set/sum/setsum)."""
    if isinstance(expr, (int, float)):
        expr = constant(expr, dst.shape)
    if tune and op in ("set", "sum", "setsum"):
        from . import tune as _tune
        ctx = IrContext()
        if op == "sum":
            dtype, shape = dst if isinstance(dst, tuple) else ("f64", ())
        else:
            dtype, shape = dst.dtype, (dst.shape if dst.shape != (1,) or expr.shape == (1,) else ())
        ir = plan_text(dtype, shape, op, expr, ctx)
        math, contract = low.get("math", 0), low.get("contract", -1)
        best = _tune.tuned(ir, math, contract)
        if best is None:
            base = {k: v for k, v in low.items() if k in ("math", "contract")}

            def make(**cand):
                return prepare(dst, expr, op=op, n=n, sample_offset=sample_offset, reduce_out=reduce_out,
                               workspace=workspace, **base, **cand)
            best, _ = _tune.tune(make, ir, math, contract)
        low = dict(low)
        low.update(best)
    ctx = IrContext()
    if op in ("sum",):
        dtype, shape = dst if isinstance(dst, tuple) else ("f64", ())
        ir = plan_text(dtype, shape, op, expr, ctx)
        n = int(n)
        return Launch(get_plan(ir, **low), ctx, n, 0, 0, sample_offset, reduce_out.data_ptr(), workspace)
    n = dst.n if n is None else int(n)
    ir = plan_text(dst.dtype, dst.shape if dst.shape != (1,) or expr.shape == (1,) else (), op, expr, ctx)
    red = reduce_out.data_ptr() if reduce_out is not None else None
    return Launch(get_plan(ir, **low), ctx, n, dst.data.data_ptr(), dst.capacity, sample_offset, red, workspace)


def assign(dst, expr, op="set", stream=None, **kw):
    """dst[i] = expr for every sample i, in one kernel (expr/Assign.h:251-346)."""
    L = prepare(dst, expr, op=op, **kw)
    L(stream)
    return dst


def assign_add(dst, expr, **kw):
    return assign(dst, expr, op="add", **kw)


def assign_sub(dst, expr, **kw):
    return assign(dst, expr, op="sub", **kw)


def global_sum(expr, n, dtype="f64", stream=None, workspace=None, **kw):
    """Compensated sum over samples of a rank-0 expression: returns a device
    tensor (hi, comp), reduced in a fixed order (deterministic)."""
    torch = _torch()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    L = prepare((dtype, ()), expr, op="sum", n=n, reduce_out=out, workspace=workspace, **kw)
    L(stream)
    return out


def _stream(stream):
    return ctypes.c_void_p(stream if stream is not None else _torch().cuda.current_stream().cuda_stream)


class Batch:
    """Many assignments in one persistent launch (aether_batch_*).

    `launches` is a list of Launch objects (from prepare()); their plans are
    grouped, one kernel is generated for the distinct plans, and the work list
    holds one argument block per launch."""

    def __init__(self, launches, block=0, ipt=0):
        plans, index = [], {}
        for L in launches:
            h = L.plan.handle.value
            if h not in index:
                index[h] = len(plans)
                plans.append(L.plan)
        self._plans = plans
        self._launches = list(launches)
        arr = (ctypes.c_void_p * len(plans))(*[p.handle for p in plans])
        h = ctypes.c_void_p()
        low = lowering(block, ipt)
        _abi.check(_abi.lib().aether_batch_create(arr, len(plans), ctypes.byref(low), ctypes.byref(h)))
        self.handle = h
        items = (_abi.AetherBatchItem * max(1, len(launches)))()
        for i, L in enumerate(launches):
            items[i].plan = index[L.plan.handle.value]
            items[i].args = L.args
        self._items = items
        _abi.check(_abi.lib().aether_batch_set_items(self.handle, items, len(launches), _stream(None)))

    def launch(self, stream=None):
        _abi.check(_abi.lib().aether_batch_launch(self.handle, _stream(stream)))

    def capture(self, stream):
        """Capture one launch into a CUDA graph on `stream` (a non-default
        stream handle, e.g. torch.cuda.Stream().cuda_stream)."""
        _abi.check(_abi.lib().aether_batch_capture(self.handle, ctypes.c_void_p(stream)))

    def replay(self, stream=None):
        _abi.check(_abi.lib().aether_batch_replay(self.handle, _stream(stream)))

    def info(self):
        i = _abi.AetherBatchInfo()
        _abi.check(_abi.lib().aether_batch_info(self.handle, ctypes.byref(i)))
        return i

    def launch_each(self, stream=None):
        """The per-call baseline: one plain launch per item from a C loop."""
        n = len(self._launches)
        plans = (ctypes.c_void_p * n)(*[L.plan.handle for L in self._launches])
        args = (_abi.AetherLaunch * n)(*[L.args for L in self._launches])
        _abi.check(_abi.lib().aether_plan_launch_many(plans, args, n, _stream(stream)))

    def __del__(self):
        try:
            if self.handle:
                _abi.lib().aether_batch_release(self.handle)
        except Exception:
            pass


from .runtime import RuntimeOp, runtime_eval, runtime_view  # noqa: E402

__all__ = [
    "Batch", "RuntimeOp", "runtime_eval", "runtime_view", "padded_block_samples", "partition_view", "AccumPlane",
    "pinned_empty",
    "Array", "Plan", "Launch", "AetherError", "Generator", "Expr", "assign", "assign_add", "assign_sub", "global_sum",
    "prepare", "get_plan", "quantized_capacity", "constant", "literal", "stack", "select", "clamp", "cwiseAbs",
    "cwiseAcos", "cwiseAsin", "cwiseAtan", "cwiseCbrt", "cwiseCeil", "cwiseCos", "cwiseCosh", "cwiseDiv", "cwiseErf",
    "cwiseExp", "cwiseExp2", "cwiseExpm1", "cwiseFloor", "cwiseLog", "cwiseLog10", "cwiseLog1p", "cwiseLog2",
    "cwiseMul", "cwiseSinh", "cwiseTrunc",
    "cwiseMax", "cwiseMin", "cwisePow", "cwiseRsqrt", "cwiseSign", "cwiseSin", "cwiseSqrt", "cwiseSquare", "cwiseTan",
    "cwiseTanh", "splitmix64", "lowering",
]
