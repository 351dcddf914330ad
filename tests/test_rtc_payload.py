"""The NVRTC payload: the device headers are exported by name with a stable
digest, can be served to a private directory and removed, and a kernel
written outside the engine (as a code generator would) that calls the
Philox stream, the double-float sine and the compensated-sum primitives
compiles against them with NVRTC for sm_103a."""

import os

import pytest

from aether_gb300 import rtc

HAWK_STYLE_KERNEL = r'''
#include "ag_device.cuh"
#include "ag_emu64.cuh"
extern "C" __global__ void user_kernel(double* out, unsigned long long key, unsigned n) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ag::q4 w = ag::philox_block(key, i, 0u);
    bool ok = true;
    const ag::e64::df x = ag::e64::scale(ag::e64::from_u64(2ull * w.x + 1ull), ag::e64::p2f(-33));
    const ag::e64::df s = ag::e64::sin_(x, ok);
    double h = 0.0, c = 0.0;
    ag::neumaier_add(h, c, ag::e64::to_double(s));
    out[i] = ok ? h + c : ag::f_sin((double)x.hi + (double)x.lo);
}
'''


def test_payload_headers_and_digest():
    p = rtc.payload()
    assert set(p.headers) == {"ag_device.cuh", "ag_emu64.cuh", "ag_emu64_tables.cuh", "ag_emu64_bm.cuh",
                              "ag_emu64_bm_tables.cuh"}
    assert all(len(v) > 1000 for v in p.headers.values())
    assert len(p.digest) == 16 and rtc.payload().digest == p.digest


def test_payload_serve_is_private_and_removed():
    p = rtc.payload()
    with p.serve() as d:
        assert oct(os.stat(d).st_mode & 0o777) == "0o700"
        for name, src in p.headers.items():
            assert open(os.path.join(d, name), "rb").read() == src
    assert not os.path.exists(d)


def test_generated_style_kernel_compiles_against_the_payload():
    rtc.compile_check(HAWK_STYLE_KERNEL)
    with pytest.raises(Exception, match="NVRTC"):
        rtc.compile_check(HAWK_STYLE_KERNEL.replace("ag::e64::sin_(x, ok)", "ag::e64::no_such_function(x)"))
