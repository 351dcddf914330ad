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


RUNTIME = ["ag_device.cuh", "ag_emu64.cuh", "ag_emu64_tables.cuh", "ag_emu64_bm.cuh", "ag_emu64_bm_tables.cuh",
           "ag_tf64.cuh", "ag_tf64_tables.cuh", "ag_tf64_trig.cuh", "ag_tf64_trig_tables.cuh"]
CONSUMER = ["aether/macros.h", "aether/detail/std.h", "aether/layout.h", "aether/math.h", "aether/expression.h",
            "aether/nodes.h", "aether/geometry.h", "aether/view.h", "aether/item.h", "aether/bundle.h", "aether/detail/philox.h",
            "aether/random.h", "aether/device.h"]

# A kernel in the reference's consumer spelling, as a code generator emits it
# against aether/device.h: typed views, SampleIndex, view[i] = expr, an Item,
# aether::math and a random leaf.
DEVICE_H_KERNEL = r'''
#include "aether/device.h"
using V3 = aether::View<double, aether::extents<3, aether::dyn>, aether::layout_stride>;
extern "C" __global__ void generated(V3 a, V3 b, V3 d, aether::random::Generator g) {
    const aether::SampleIndex i = aether::SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
    if (i.global() >= d.samples()) return;
    a[i] = g.substream(0).uniform<double, 3>(-1.0, 1.0);
    const aether::Vec3d x = a[i].get();
    const aether::Vec3d s{aether::math::sin(x(0)), aether::math::sin(x(1)), aether::math::sin(x(2))};
    d[i] = a.cross(b) + s * aether::cwiseExp(b * (-1.0));
}
'''


def test_payload_headers_and_digest():
    p = rtc.payload()
    assert set(p.headers) == set(RUNTIME) | set(CONSUMER) | {"aether/gb300/" + n for n in RUNTIME}
    assert all(len(v) > 300 for v in p.headers.values())
    assert p.headers["aether/gb300/ag_emu64.cuh"] == p.headers["ag_emu64.cuh"]
    assert len(p.digest) == 16 and rtc.payload().digest == p.digest
    # the payload is the consumer headers of the source tree, byte for byte
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    for name in CONSUMER:
        assert open(os.path.join(inc, name), "rb").read() == p.headers[name], name


def test_device_h_kernel_compiles_with_nvrtc():
    for opts in ([], ["-DAETHER_GB300_EMULATED_FP64"], ["-DAETHER_GB300_FP64_GRADE"], ["--fmad=false"]):
        cubin = rtc.compile(DEVICE_H_KERNEL, options=opts)
        assert len(cubin) > 1000 and cubin[:4] == b"\x7fELF"
    with pytest.raises(Exception, match="NVRTC"):
        rtc.compile(DEVICE_H_KERNEL.replace("a.cross(b)", "a.no_such_member(b)"))


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


@pytest.mark.gpu
def test_device_h_kernel_runs_through_the_driver_api(tmp_path, oracle):
    """A generated kernel compiled by aether_rtc_compile, loaded with the
    driver API and launched on aether::Array views: its Philox draws equal the
    oracle's and its arithmetic is bit-exact with contraction off."""
    import shutil
    import subprocess

    import numpy as np

    from aether_gb300 import build
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cuda = build.cuda_home()
    libdir = os.path.join(repo, "aether_gb300", "lib")
    exe = str(tmp_path / "rtc_consumer")
    cmd = [shutil.which("g++"), "-std=c++17", "-O1", "-I", os.path.join(repo, "include"),
           "-I", os.path.join(cuda, "include"), os.path.join(repo, "tests", "cpp", "rtc_consumer.cpp"), "-o", exe,
           "-L", libdir, "-laether_gb300", "-Wl,-rpath," + libdir]
    # link the driver API through the toolkit's stub (the driver's libcuda.so.1 loads at run time)
    for stub in (os.path.join(cuda, "lib64", "stubs"), os.path.join(cuda, "lib", "stubs")):
        if os.path.exists(os.path.join(stub, "libcuda.so")):
            cmd += ["-L", stub]
    cmd.append("-lcuda")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n = 4099
    out = tmp_path / "rtc.bin"
    run = subprocess.run([exe, str(out), str(n), rtc.libcudacxx_include()], capture_output=True, text=True,
                         timeout=300)
    assert run.returncode == 0 and "rtc consumer ok" in run.stdout, run.stdout + run.stderr
    cap = (n + 31) // 32 * 32
    a, b, d = (np.ascontiguousarray(x[:, :n]) for x in np.fromfile(str(out), dtype=np.float64).reshape(3, 3, cap))
    k42 = oracle.generator_key(42)
    assert np.array_equal(a, oracle.fill_uniform_f64(oracle.substream_key(k42, 0), -1.0, 1.0, 3, n))
    assert np.array_equal(b, oracle.fill_uniform_f64(oracle.substream_key(k42, 1), -1.0, 1.0, 3, n))
    cross = np.stack([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])
    assert np.array_equal(d, cross + a * b)
