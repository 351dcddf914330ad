"""The seam table on the device (dsc/src/seam.h:22-53 behaviour): a device
chunk allocated through aether_memory_v1, filled with a multi-byte pattern,
copied to pinned memory, its owning device reported, then released."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_seam_table_round_trip():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from aether_gb300 import _abi
    L = _abi.lib()
    P = ctypes.c_void_p
    chunk, ptr, hchunk, hptr = P(), P(), P(), P()
    n = 1000
    _abi.check(L.aether_chunk_alloc(1, 0, n * 8, None, ctypes.byref(chunk), ctypes.byref(ptr)))
    _abi.check(L.aether_chunk_alloc(2, 0, n * 8, None, ctypes.byref(hchunk), ctypes.byref(hptr)))
    pattern = np.array([1.25], dtype=np.float64)
    _abi.check(L.aether_fill(1, 0, ptr, n * 8, pattern.ctypes.data, 8, None))
    _abi.check(L.aether_copy(2, 0, hptr, 1, 0, ptr, n * 8, None))
    _abi.check(L.aether_stream_sync(0, None))
    host = np.ctypeslib.as_array(ctypes.cast(hptr, ctypes.POINTER(ctypes.c_double)), shape=(n,))
    assert np.all(host == 1.25)
    dev, cur = ctypes.c_int(-1), ctypes.c_int(-1)
    _abi.check(L.aether_pointer_device(ptr, ctypes.byref(dev)))
    _abi.check(L.aether_current_device(ctypes.byref(cur)))
    assert dev.value == cur.value == torch.cuda.current_device()
    assert L.aether_pointer_device(hptr, ctypes.byref(dev)) == 1     # pinned host memory is not a device pointer
    L.aether_chunk_release(chunk)
    L.aether_chunk_release(hchunk)
    L.aether_drain()


def test_pinned_empty_is_registered_and_round_trips():
    """Host chunks of kind 2 back ag.pinned_empty: page-locked, copied by the
    copy engines, and released with the last view."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import aether_gb300 as ag
    from aether_gb300 import _abi
    L = _abi.lib()
    h = ag.pinned_empty((3, 1000))
    h.copy_(torch.arange(3000, dtype=torch.float64).reshape(3, 1000))
    dev = torch.empty((3, 1000), dtype=torch.float64, device="cuda")
    P = ctypes.c_void_p
    _abi.check(L.aether_copy(1, 0, P(dev.data_ptr()), 2, 0, P(h.data_ptr()), 3000 * 8, None))
    _abi.check(L.aether_stream_sync(0, None))
    assert torch.equal(dev.cpu(), h)
    d = ctypes.c_int(-1)
    assert L.aether_pointer_device(P(h.data_ptr()), ctypes.byref(d)) == 1   # host memory, not a device pointer
    del h
