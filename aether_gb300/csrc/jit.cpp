// jit.cpp -- NVRTC front of the plan cache.
//
// The reference compiles one kernel per consumer expression with nvcc, or
// lets hawk compile the sealed headers with NVRTC (tools/nvrtc/README.md).
// Here the engine itself generates the kernel text from the plan and
// compiles it for the device it runs on; the device headers are embedded in
// the library, so nothing is read from disk at run time except the cache.

#include "jit.h"

#include <cuda_runtime.h>
#include <nvrtc.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <sys/stat.h>
#include <unistd.h>
#include <unordered_map>

#include "embedded.inc"   // kAgDeviceSrc, kAgEmu64Src

namespace ag {

uint64_t fnv1a(const std::string& s, uint64_t h) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ULL;
    }
    return h;
}

std::string current_arch() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) throw std::runtime_error("cudaGetDevice failed");
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major < 10)
        throw std::runtime_error("aether_gb300 targets Blackwell (sm_103a); device " + std::to_string(dev) +
                                 " is sm_" + std::to_string(major) + std::to_string(minor));
    return "sm_" + std::to_string(major) + std::to_string(minor) + "a";
}

namespace {

std::string cache_dir() {
    if (const char* d = std::getenv("AETHER_GB300_CACHE")) return d;
    if (const char* x = std::getenv("XDG_CACHE_HOME")) return std::string(x) + "/aether_gb300";
    if (const char* h = std::getenv("HOME")) return std::string(h) + "/.cache/aether_gb300";
    return "/tmp/aether_gb300_cache";
}

void mkdirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur += path[i];
        if (path[i] == '/' && cur.size() > 1) ::mkdir(cur.c_str(), 0755);
    }
    ::mkdir(path.c_str(), 0755);
}

bool read_file(const std::string& p, std::string& out) {
    std::ifstream f(p, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return !out.empty();
}

std::mutex g_mu;
std::unordered_map<uint64_t, std::string> g_mem;

}  // namespace

int payload_count() { return 5; }

bool payload_header(int i, const char** name, const char** src) {
    static const char* const names[] = {"ag_device.cuh", "ag_emu64.cuh", "ag_emu64_tables.cuh", "ag_emu64_bm.cuh",
                                        "ag_emu64_bm_tables.cuh"};
    static const char* const srcs[] = {kAgDeviceSrc, kAgEmu64Src, kAgEmu64TablesSrc, kAgEmu64BmSrc,
                                       kAgEmu64BmTablesSrc};
    if (i < 0 || i >= 5) return false;
    *name = names[i];
    *src = srcs[i];
    return true;
}

uint64_t payload_digest() {
    uint64_t h = fnv1a(std::string("aether_gb300 rtc payload"));
    for (int i = 0; i < payload_count(); ++i) {
        const char *n = nullptr, *s = nullptr;
        payload_header(i, &n, &s);
        h = fnv1a(n, h);
        h = fnv1a(s, h);
    }
    return h;
}

std::string compile_for_arch(const std::string& source, const std::string& arch) {
    const char* hdr_src[] = {kAgDeviceSrc, kAgEmu64Src, kAgEmu64TablesSrc, kAgEmu64BmSrc, kAgEmu64BmTablesSrc};
    const char* hdr_names[] = {"ag_device.cuh", "ag_emu64.cuh", "ag_emu64_tables.cuh", "ag_emu64_bm.cuh",
                               "ag_emu64_bm_tables.cuh"};
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, source.c_str(), "aether_plan.cu", 5, hdr_src, hdr_names) != NVRTC_SUCCESS)
        throw std::runtime_error("nvrtcCreateProgram failed");
    const std::string arch_opt = "--gpu-architecture=" + arch;
    const char* opts[] = {arch_opt.c_str(), "--std=c++17", "--fmad=true", "--dopt=on"};
    const nvrtcResult rc = nvrtcCompileProgram(prog, 4, opts);
    if (rc != NVRTC_SUCCESS) {
        size_t n = 0;
        nvrtcGetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) nvrtcGetProgramLog(prog, &log[0]);
        nvrtcDestroyProgram(&prog);
        throw std::runtime_error(std::string("NVRTC compile failed (") + nvrtcGetErrorString(rc) + "):\n" + log);
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    std::string cubin(n, '\0');
    nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    return cubin;
}

Compiled compile_cached(const std::string& source, const std::string& tag) {
    const std::string arch = current_arch();
    int nvrtc_major = 0, nvrtc_minor = 0;
    nvrtcVersion(&nvrtc_major, &nvrtc_minor);
    const std::string opts_key = arch + "|nvrtc" + std::to_string(nvrtc_major) + "." + std::to_string(nvrtc_minor) + "|" + tag;
    uint64_t h = fnv1a(source);
    h = fnv1a(opts_key, h);
    h = fnv1a(kAgDeviceSrc, h);
    h = fnv1a(kAgEmu64Src, h);
    h = fnv1a(kAgEmu64TablesSrc, h);

    Compiled out;
    out.hash = h;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_mem.find(h);
        if (it != g_mem.end()) {
            out.cubin = it->second;
            return out;
        }
    }
    char name[32];
    std::snprintf(name, sizeof name, "%016llx", (unsigned long long)h);
    const std::string dir = cache_dir();
    const std::string path = dir + "/" + name + ".cubin";
    if (std::getenv("AETHER_GB300_NO_DISK_CACHE") == nullptr && read_file(path, out.cubin)) {
        std::lock_guard<std::mutex> lk(g_mu);
        g_mem[h] = out.cubin;
        return out;
    }

    const auto t0 = std::chrono::steady_clock::now();
    out.cubin = compile_for_arch(source, arch);
    out.compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();

    if (std::getenv("AETHER_GB300_NO_DISK_CACHE") == nullptr) {
        mkdirs(dir);
        const std::string tmp = path + ".tmp" + std::to_string(::getpid());
        {
            std::ofstream f(tmp, std::ios::binary);
            f.write(out.cubin.data(), std::streamsize(out.cubin.size()));
        }
        std::rename(tmp.c_str(), path.c_str());
    }
    std::lock_guard<std::mutex> lk(g_mu);
    g_mem[h] = out.cubin;
    return out;
}

}  // namespace ag
