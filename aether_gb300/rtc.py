"""The NVRTC payload (aether_rtc_*): the device headers generated kernels
include, for kernels a code generator compiles with its own NVRTC program.

The counterpart of the reference's sealed header payload
(dsc/aether_dsc/_core.py:132-200): `payload()` returns the headers by
include name with a content digest; `Payload.serve()` materialises them in a
private directory for the lifetime of a `with` block (for compilers that
read include directories rather than in-memory headers).
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
                with open(os.path.join(d, name), "wb") as f:
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
