"""The NVRTC payload (aether_rtc_*): the device-safe consumer headers
(aether/device.h and what it includes) and the engine's device runtime, for
kernels a code generator compiles with NVRTC.

The counterpart of the reference's sealed header payload
(dsc/aether_dsc/_core.py:132-200): `payload()` returns the headers by
include name with a content digest; `Payload.serve()` materialises them in a
private directory for the lifetime of a `with` block (for compilers that
read include directories rather than in-memory headers); `compile()` runs
NVRTC over a source against the payload and returns the CUBIN.
"""

import contextlib
import ctypes
import os
import shutil
import tempfile

from . import _abi


class Payload:
    __slots__ = ("digest", "headers")

    def __init__(self, digest, headers):
        self.digest = digest
        self.headers = dict(headers)

    @contextlib.contextmanager
    def serve(self):
        d = tempfile.mkdtemp(prefix="aether_gb300_rtc_")
        try:
            os.chmod(d, 0o700)
            for name, src in self.headers.items():
                path = os.path.join(d, name)
                os.makedirs(os.path.dirname(path), mode=0o700, exist_ok=True)
                with open(path, "wb") as f:
                    f.write(src)
            yield d
        finally:
            shutil.rmtree(d, ignore_errors=True)


def payload():
    L = _abi.lib()
    headers = {}
    for i in range(L.aether_rtc_header_count()):
        name, src = ctypes.c_char_p(), ctypes.c_char_p()
        _abi.check(L.aether_rtc_header(i, ctypes.byref(name), ctypes.byref(src)))
        headers[name.value.decode()] = src.value
    return Payload("%016x" % L.aether_rtc_digest(), headers)


def compile_check(source, arch="sm_103a"):
    """NVRTC-compile a kernel that includes the payload headers (no load)."""
    _abi.nvrtc_check(source, arch)


def libcudacxx_include():
    """The CUDA toolkit directory that holds libcu++ (cuda/std/...), which the
    consumer headers use under NVRTC."""
    from . import build
    home = build.cuda_home()
    for cand in (os.path.join(home, "include", "cccl"), os.path.join(home, "include")):
        if os.path.isdir(os.path.join(cand, "cuda", "std")):
            return cand
    raise RuntimeError("libcu++ (cuda/std) not found under " + home)


def compile(source, arch="sm_103a", options=()):
    """NVRTC-compile `source` against the payload; returns the CUBIN bytes.
    The libcu++ include path is added for aether/device.h."""
    L = _abi.lib()
    opts = ["--include-path=" + libcudacxx_include()] + list(options)
    arr = (ctypes.c_char_p * len(opts))(*[o.encode() for o in opts])
    n = ctypes.c_size_t()
    _abi.check(L.aether_rtc_compile(source.encode(), arch.encode(), arr, len(opts), None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value)
    _abi.check(L.aether_rtc_compile(source.encode(), arch.encode(), arr, len(opts), buf, n.value, ctypes.byref(n)))
    return buf.raw[: n.value]
