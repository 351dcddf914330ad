"""In-tree build of libaether_gb300.so (the C-ABI engine).

Host sources compile with g++, device sources with nvcc for sm_103a only; the
device headers that generated kernels include are embedded as string
literals. Translation units compile in parallel; nothing here needs cmake.

usage: python -m aether_gb300.build [--force]
"""

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libaether_gb300.so")
# The same objects linked as the reference's CUDA plugin: exactly one exported
# symbol, aether_memory_v1 (dsc/src/plugin.map:1-4), under the file name the
# reference's loader opens next to its module (dsc/src/aether_core.cpp:98-101).
PLUGIN = os.path.join(LIBDIR, "libaether_cuda.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

HOST_SOURCES = ["plan.cpp", "jit.cpp", "abi.cpp", "serve.cpp", "tables.cpp"]
DEVICE_SOURCES = ["noalloc.cu", "runtime.cu", "serve_copy.cu"]
# The device runtime headers live in the public include tree (consumer kernels
# compiled with nvcc include them too); generated kernels get them embedded.
DEVICE_INC = os.path.join(REPO, "include", "aether", "gb300")
EMBED = [("kAgDeviceSrc", "ag_device.cuh"), ("kAgEmu64Src", "ag_emu64.cuh"),
         ("kAgEmu64TablesSrc", "ag_emu64_tables.cuh"), ("kAgEmu64BmSrc", "ag_emu64_bm.cuh"),
         ("kAgEmu64BmTablesSrc", "ag_emu64_bm_tables.cuh"), ("kAgTf64Src", "ag_tf64.cuh"),
         ("kAgTf64TablesSrc", "ag_tf64_tables.cuh"), ("kAgTf64TrigSrc", "ag_tf64_trig.cuh"),
         ("kAgTf64TrigTablesSrc", "ag_tf64_trig_tables.cuh")]
# The device-safe consumer headers (aether/device.h and what it includes),
# exported with the engine's device runtime as the NVRTC payload for code
# generators, each under its include name.
CONSUMER_HEADERS = ["macros.h", "detail/std.h", "layout.h", "math.h", "expression.h", "nodes.h", "geometry.h",
                    "view.h", "item.h", "bundle.h", "detail/philox.h", "random.h", "device.h"]
EXPORT_PREFIX = "aether_"


def cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _write_if_changed(path, text):
    if os.path.exists(path) and open(path).read() == text:
        return
    with open(path, "w") as f:
        f.write(text)


def _embed():
    parts = ["// generated by aether_gb300/build.py from include/aether/gb300/*.cuh\n"]
    for name, rel in EMBED:
        src = open(os.path.join(DEVICE_INC, rel)).read()
        delim = "AGSRC"
        assert ")" + delim + '"' not in src
        # Raw literals are limited in length by some compilers: split in pieces.
        pieces = [src[i:i + 12000] for i in range(0, len(src), 12000)] or [""]
        body = "\n".join('R"%s(%s)%s"' % (delim, p, delim) for p in pieces)
        parts.append("static const char* const %s =\n%s;\n" % (name, body))
    table = []
    for k, rel in enumerate(CONSUMER_HEADERS):
        src = open(os.path.join(REPO, "include", "aether", rel)).read()
        delim = "AGSRC"
        assert ")" + delim + '"' not in src
        pieces = [src[i:i + 12000] for i in range(0, len(src), 12000)] or [""]
        body = "\n".join('R"%s(%s)%s"' % (delim, p, delim) for p in pieces)
        parts.append("static const char* const kConsumer%d =\n%s;\n" % (k, body))
        table.append('    {"aether/%s", kConsumer%d},\n' % (rel, k))
    parts.append("struct AgNamedSource {\n    const char* name;\n    const char* src;\n};\n")
    parts.append("static const AgNamedSource kConsumerHeaders[] = {\n%s};\n" % "".join(table))
    _write_if_changed(os.path.join(BUILD, "embedded.inc"), "".join(parts))


def _exports():
    text = "{\n  global: %s*;\n  local: *;\n};\n" % EXPORT_PREFIX
    _write_if_changed(os.path.join(BUILD, "exports.map"), text)
    _write_if_changed(os.path.join(BUILD, "plugin.map"), "{\n  global: aether_memory_v1;\n  local: *;\n};\n")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    out = []
    for top in (CSRC, os.path.join(REPO, "include", "aether")):
        for root, _, files in os.walk(top):
            out += [os.path.join(root, f) for f in files if f.endswith((".h", ".cuh", ".inc"))]
    out.append(os.path.join(REPO, "include", "aether_gb300.h"))
    out.append(os.path.join(BUILD, "embedded.inc"))
    return out


def build(force=False, verbose=False):
    cuda = cuda_home()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    _embed()
    _exports()
    inc = ["-I" + os.path.join(REPO, "include"), "-I" + DEVICE_INC, "-I" + CSRC, "-I" + BUILD,
           "-I" + os.path.join(cuda, "include")]
    hdrs = _headers()
    jobs = []
    objs = []
    for s in HOST_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wno-unused-function",
                         "-c", src, "-o", obj] + inc)
    for s in DEVICE_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([os.path.join(cuda, "bin", "nvcc"), ARCH, "-O3", "-std=c++17", "-lineinfo",
                         "-Xcompiler", "-fPIC,-fvisibility=hidden", "-c", src, "-o", obj] + inc)
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
        for j, f in zip(jobs, futs):
            r = f.result()
            if verbose or r.returncode:
                sys.stderr.write(" ".join(j) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("compile failed: " + j[-len(inc) - 1 if False else 0] + " " + " ".join(j[:6]))
    if force or jobs or not os.path.exists(LIB) or not os.path.exists(PLUGIN):
        libdir = os.path.join(cuda, "lib64")
        if not os.path.isdir(libdir):
            libdir = os.path.join(cuda, "lib")
        links = []
        for out, vmap in ((LIB, "exports.map"), (PLUGIN, "plugin.map")):
            links.append(["g++", "-shared", "-o", out] + objs + [
                "-L" + libdir, "-lcudart_static", "-lnvrtc", "-ldl", "-lpthread", "-lrt",
                "-Wl,-rpath," + libdir, "-Wl,--version-script=" + os.path.join(BUILD, vmap),
                "-Wl,--no-undefined"])
        with cf.ThreadPoolExecutor(max_workers=2) as ex:
            for cmd, r in zip(links, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), links)):
                if r.returncode:
                    raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
