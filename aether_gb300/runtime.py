"""Runtime-typed strided evaluation (aether_runtime_eval).

The Python face of aether::eval::runtimeEval (eval/Runtime.h:73-300): torch
tensors of any strides (float32 or float64, on the device) stand in for the
reference's RuntimeView descriptors (view/RuntimeView.h:71-110), whose fields
a tensor carries as (data_ptr, dtype, shape, stride) -- the DLPack fields.

    runtime_eval(RuntimeOp.AddScaled, a, b, out, scalar=0.5)   # out = a + 0.5*b
"""

import ctypes

from . import _abi


class RuntimeOp:
    Assign = 0
    Add = 1
    Sub = 2
    Scale = 3
    AddScaled = 4
    SubScaled = 5


_DT = {"torch.float64": (2, 64), "torch.float32": (2, 32), "torch.int32": (0, 32), "torch.int64": (0, 64),
       "torch.float16": (2, 16), "torch.bfloat16": (4, 16)}


def runtime_view(t):
    """An AetherRuntimeView over a tensor's storage (no copy)."""
    if t.dim() > 6:
        raise _abi.AetherError("aether runtime views hold rank <= 6 (got %d)" % t.dim())
    v = _abi.AetherRuntimeView()
    v.data = t.data_ptr()
    code, bits = _DT.get(str(t.dtype), (255, 0))
    v.dtype_code, v.dtype_bits, v.dtype_lanes = code, bits, 1
    v.rank = t.dim()
    for k, (e, s) in enumerate(zip(t.shape, t.stride())):
        v.extents[k] = int(e)
        v.strides[k] = int(s)
    return v


def runtime_eval(op, a, b, out, scalar=0.0, stream=None):
    """out = op(a, b, scalar) elementwise, one kernel on `stream` (default:
    torch's current stream). b may be None for Assign and Scale."""
    import torch
    va, vo = runtime_view(a), runtime_view(out)
    vb = runtime_view(b) if b is not None else None
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream if torch.cuda.is_available() else 0
    s = stream
    _abi.check(_abi.lib().aether_runtime_eval(int(op), ctypes.byref(va), ctypes.byref(vb) if vb is not None else None,
                                              ctypes.byref(vo), float(scalar), ctypes.c_void_p(s)))
    return out
