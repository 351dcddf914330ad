"""aether::interop's C++ DLPack import and export (include/aether/dlpack.h;
interop/DLPack.h:226-430 and interop/DLPackLegacy.h) and its buffer layer
(include/aether/buffer.h; interop/Buffer.h).

CPU: tests/cpp/dlpack_interop.cpp, the reference's import, refusal and
round-trip cases (tests/test_DLPackRoundtrip.cu, tests/test_DLPackDtypes_common.h),
and tests/cpp/buffer_interop.cpp, the buffer layer's (aether/buffer.h,
tests/test_DLPackBuffer_common.h), over producers whose deleters count their
calls, run under the address and
undefined-behaviour sanitizers; the same source against the DLPack project's
own header as torch ships it, whose struct layout must equal ours byte for
byte; the header in a CUDA translation unit.
GPU: torch as the foreign producer, both DLPack generations, its tensors
imported by the C++ interop and scaled by the engine's runtime evaluation."""

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(REPO, "aether_gb300", "lib")
SRC = os.path.join(REPO, "tests", "cpp", "dlpack_interop.cpp")
BUFFER_SRC = os.path.join(REPO, "tests", "cpp", "buffer_interop.cpp")


def _cxx():
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    return cxx


def _torch_include():
    torch = pytest.importorskip("torch")
    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    if not os.path.exists(os.path.join(inc, "ATen", "dlpack.h")):
        pytest.skip("torch ships no dlpack.h")
    return inc


def _build_and_run(tmp_path, name, extra, src=SRC, ok="dlpack ok"):
    exe = str(tmp_path / name)
    r = subprocess.run([_cxx(), "-std=c++17", "-O1", "-g", "-Wall", "-Wextra", "-I", INCLUDE, src, "-o", exe] + extra,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0 and ok in run.stdout, run.stdout + run.stderr


def _sanitizers(tmp_path):
    probe = subprocess.run([_cxx(), "-fsanitize=address,undefined", "-x", "c++", "-", "-o", str(tmp_path / "p")],
                           input="int main(){}", capture_output=True, text=True)
    return ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"] if probe.returncode == 0 else []


def test_interop_cases_under_sanitizers(tmp_path):
    _build_and_run(tmp_path, "dlpack_interop", _sanitizers(tmp_path))


def test_interop_cases_against_the_projects_header(tmp_path):
    inc = _torch_include()
    _build_and_run(tmp_path, "dlpack_interop_torch", ["-I", inc, "-include", "ATen/dlpack.h"])


def test_buffer_layer_under_sanitizers(tmp_path):
    """aether/buffer.h (interop/Buffer.h): access from both DLPack generations
    and the array interface, keep-alive chains, requirements and their
    messages, exports that carry the read-only flag
    (tests/test_DLPackBuffer_common.h)."""
    _build_and_run(tmp_path, "buffer_interop", _sanitizers(tmp_path), BUFFER_SRC, "buffer ok")


def test_buffer_layer_against_the_projects_header(tmp_path):
    inc = _torch_include()
    _build_and_run(tmp_path, "buffer_interop_torch", ["-I", inc, "-include", "ATen/dlpack.h"], BUFFER_SRC, "buffer ok")


LAYOUT = r"""
#include <cstddef>
#include <cstdio>
%s
#define P(T, F) std::printf(#T "." #F " %%zu\n", offsetof(T, F))
#define S(T) std::printf(#T " %%zu %%zu\n", sizeof(T), alignof(T))
int main() {
    S(DLPackVersion); S(DLDevice); S(DLDataType); S(DLTensor); S(DLManagedTensor); S(DLManagedTensorVersioned);
    P(DLDevice, device_id); P(DLDataType, bits); P(DLDataType, lanes);
    P(DLTensor, data); P(DLTensor, device); P(DLTensor, ndim); P(DLTensor, dtype); P(DLTensor, shape);
    P(DLTensor, strides); P(DLTensor, byte_offset);
    P(DLManagedTensor, dl_tensor); P(DLManagedTensor, manager_ctx); P(DLManagedTensor, deleter);
    P(DLManagedTensorVersioned, version); P(DLManagedTensorVersioned, manager_ctx);
    P(DLManagedTensorVersioned, deleter); P(DLManagedTensorVersioned, flags); P(DLManagedTensorVersioned, dl_tensor);
    std::printf("kDLCPU %%d kDLCUDA %%d kDLCUDAHost %%d kDLOpenCL %%d kDLROCMHost %%d kDLCUDAManaged %%d\n",
                int(kDLCPU), int(kDLCUDA), int(kDLCUDAHost), int(kDLOpenCL), int(kDLROCMHost), int(kDLCUDAManaged));
    std::printf("kDLInt %%d kDLUInt %%d kDLFloat %%d kDLBfloat %%d kDLComplex %%d kDLBool %%d\n",
                int(kDLInt), int(kDLUInt), int(kDLFloat), int(kDLBfloat), int(kDLComplex), int(kDLBool));
}
"""


def _layout(tmp_path, name, include_lines, extra):
    src = tmp_path / (name + ".cpp")
    src.write_text(LAYOUT % include_lines)
    exe = str(tmp_path / name)
    r = subprocess.run([_cxx(), "-std=c++17", "-I", INCLUDE, str(src), "-o", exe] + extra, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    return subprocess.run([exe], capture_output=True, text=True, check=True).stdout


def test_struct_layout_equals_the_projects(tmp_path):
    inc = _torch_include()
    ours = _layout(tmp_path, "ours", "#include <aether/aether.h>\n#include <aether/dlpack.h>", [])
    theirs = _layout(tmp_path, "theirs", "#include <ATen/dlpack.h>", ["-I", inc])
    assert ours == theirs
    assert "DLManagedTensorVersioned.dl_tensor" in ours


def test_header_compiles_in_a_cuda_translation_unit(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-c",
                        "-DDLPACK_WITH_ENGINE", "-I", INCLUDE, SRC, "-o", str(tmp_path / "dlpack.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


# -- GPU: torch produces, the C++ interop imports, the engine computes -------

def _capsule_pointer(cap, name):
    api = ctypes.pythonapi
    api.PyCapsule_GetPointer.restype = ctypes.c_void_p
    api.PyCapsule_GetPointer.argtypes = [ctypes.py_object, ctypes.c_char_p]
    api.PyCapsule_SetName.restype = ctypes.c_int
    api.PyCapsule_SetName.argtypes = [ctypes.py_object, ctypes.c_char_p]
    p = api.PyCapsule_GetPointer(cap, name.encode())
    # the consumer protocol: a consumed capsule is renamed, so its destructor
    # leaves the deleter to the importer
    assert api.PyCapsule_SetName(cap, ("used_" + name).encode()) == 0
    return p


def _export(t, versioned):
    if versioned:
        try:
            return _capsule_pointer(t.__dlpack__(max_version=(1, 0)), "dltensor_versioned"), 1
        except TypeError:
            pytest.skip("this torch exports no versioned DLPack tensors")
    return _capsule_pointer(t.__dlpack__(), "dltensor"), 0


@pytest.fixture(scope="module")
def scale_lib(tmp_path_factory):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import aether_gb300  # noqa: F401  (the engine library is built and loaded)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    so = str(tmp_path_factory.mktemp("dlpack") / "libdlpack_scale.so")
    r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "-shared", "-Xcompiler", "-fPIC", "-DDLPACK_WITH_ENGINE", "-I", INCLUDE, SRC, "-o", so,
                        "-L", LIBDIR, "-laether_gb300", "-Xlinker", "-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(so)
    lib.dlpack_scale.restype = ctypes.c_int
    lib.dlpack_scale.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_char_p, ctypes.c_size_t]
    return lib


def _scale(lib, x, y, s, vx, vy):
    px, fx = _export(x, vx)
    py, fy = _export(y, vy)
    err = ctypes.create_string_buffer(512)
    rc = lib.dlpack_scale(px, fx, py, fy, s, err, 512)
    return rc, err.value.decode()


@pytest.mark.gpu
@pytest.mark.parametrize("versioned", [(0, 0), (1, 1), (0, 1)])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_torch_tensors_through_the_interop(scale_lib, versioned, dtype):
    import torch
    dt = getattr(torch, dtype)
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.rand(3, 4099, generator=g, device="cuda", dtype=torch.float64).to(dt)
    y = torch.full_like(x, -1.0)
    rc, err = _scale(scale_lib, x, y, 2.5, *versioned)
    assert rc == 0, err
    assert torch.equal(y, x * 2.5)   # one IEEE product per element


@pytest.mark.gpu
def test_strided_producer_views(scale_lib):
    """A transposed input and a column-sliced output: the DLPack strides
    reach the engine unchanged, and the gaps of the output stay untouched."""
    import torch
    x = torch.arange(6 * 500, device="cuda", dtype=torch.float64).reshape(500, 6).t()   # strides (1, 6)
    base = torch.full((6, 1000), -7.0, device="cuda", dtype=torch.float64)
    y = base[:, ::2]                                                                     # strides (1000, 2)
    rc, err = _scale(scale_lib, x, y, -0.5, 0, 1)
    assert rc == 0, err
    assert torch.equal(y, x * -0.5)
    assert torch.all(base[:, 1::2] == -7.0)


@pytest.mark.gpu
def test_refused_import_reports_and_releases(scale_lib):
    import torch
    x = torch.zeros(4, 8, device="cuda", dtype=torch.complex64)
    y = torch.zeros(4, 8, device="cuda", dtype=torch.complex64)
    rc, err = _scale(scale_lib, x, y, 1.0, 0, 0)
    assert rc == 1 and "aether::interop::fromDLPack failed on DLPack" in err and "unsupported dtype" in err
    x.add_(1)   # the producer's tensors are intact after both deleters ran
    assert float(x.real.sum()) == 32.0
    assert np.isfinite(float(y.real.sum()))
