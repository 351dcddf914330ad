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
#include <vector>

#include "embedded.inc"   // kAgDeviceSrc, kAgEmu64Src, ... (the device headers as literals)

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

namespace {

// The device headers every generated kernel may include, by include name.
// One table serves the NVRTC program, the payload export and the cache key,
// so a header added here is covered by all three.
struct Header {
    const char* name;
    const char* src;
};
const Header kHeaders[] = {
    {"ag_device.cuh", kAgDeviceSrc},           {"ag_emu64.cuh", kAgEmu64Src},
    {"ag_emu64_tables.cuh", kAgEmu64TablesSrc}, {"ag_emu64_bm.cuh", kAgEmu64BmSrc},
    {"ag_emu64_bm_tables.cuh", kAgEmu64BmTablesSrc}, {"ag_tf64.cuh", kAgTf64Src},
    {"ag_tf64_tables.cuh", kAgTf64TablesSrc}, {"ag_tf64_trig.cuh", kAgTf64TrigSrc},
    {"ag_tf64_trig_tables.cuh", kAgTf64TrigTablesSrc},
};
constexpr int kNumHeaders = int(sizeof(kHeaders) / sizeof(kHeaders[0]));

}  // namespace

// The NVRTC payload: the engine's device runtime under its bare include names
// (as generated plans include it), the device-safe consumer headers under
// "aether/...", and the device runtime again under "aether/gb300/..." (as the
// consumer headers include it).
constexpr int kNumConsumer = int(sizeof(kConsumerHeaders) / sizeof(kConsumerHeaders[0]));
constexpr int kNumPayload = kNumHeaders + kNumConsumer + kNumHeaders;

namespace {
const std::string& gb300_name(int i) {
    static std::string names[kNumHeaders];
    static std::once_flag once;
    std::call_once(once, [] {
        for (int k = 0; k < kNumHeaders; ++k) names[k] = std::string("aether/gb300/") + kHeaders[k].name;
    });
    return names[i];
}
}  // namespace

int payload_count() { return kNumPayload; }

bool payload_header(int i, const char** name, const char** src) {
    if (i < 0 || i >= kNumPayload) return false;
    if (i < kNumHeaders) {
        *name = kHeaders[i].name;
        *src = kHeaders[i].src;
    } else if (i < kNumHeaders + kNumConsumer) {
        *name = kConsumerHeaders[i - kNumHeaders].name;
        *src = kConsumerHeaders[i - kNumHeaders].src;
    } else {
        const int k = i - kNumHeaders - kNumConsumer;
        *name = gb300_name(k).c_str();
        *src = kHeaders[k].src;
    }
    return true;
}

uint64_t payload_digest() {
    uint64_t h = fnv1a(std::string("aether_gb300 rtc payload"));
    for (int i = 0; i < kNumPayload; ++i) {
        const char *n = nullptr, *src = nullptr;
        payload_header(i, &n, &src);
        h = fnv1a(n, h);
        h = fnv1a(src, h);
    }
    return h;
}

uint64_t cache_key(const std::string& source, const std::string& arch, const std::string& tag, int nvrtc_major,
                   int nvrtc_minor, int override_index, const char* override_src) {
    const std::string opts_key =
        arch + "|nvrtc" + std::to_string(nvrtc_major) + "." + std::to_string(nvrtc_minor) + "|" + tag;
    uint64_t h = fnv1a(source);
    h = fnv1a(opts_key, h);
    for (int i = 0; i < kNumPayload; ++i) {
        const char *n = nullptr, *src = nullptr;
        payload_header(i, &n, &src);
        h = fnv1a(n, h);
        h = fnv1a(i == override_index && override_src ? override_src : src, h);
    }
    return h;
}

std::string compile_with_payload(const std::string& source, const std::string& arch,
                                 const std::vector<std::string>& options) {
    std::vector<const char*> srcs(kNumPayload), names(kNumPayload);
    for (int i = 0; i < kNumPayload; ++i) payload_header(i, &names[size_t(i)], &srcs[size_t(i)]);
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, source.c_str(), "aether_rtc.cu", kNumPayload, srcs.data(), names.data()) !=
        NVRTC_SUCCESS)
        throw std::runtime_error("nvrtcCreateProgram failed");
    const std::string arch_opt = "--gpu-architecture=" + arch;
    std::vector<const char*> opts = {arch_opt.c_str(), "--std=c++17"};
    for (const std::string& o : options) opts.push_back(o.c_str());
    const nvrtcResult rc = nvrtcCompileProgram(prog, int(opts.size()), opts.data());
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

std::string compile_for_arch(const std::string& source, const std::string& arch) {
    const char* hdr_src[kNumHeaders];
    const char* hdr_names[kNumHeaders];
    for (int i = 0; i < kNumHeaders; ++i) {
        hdr_src[i] = kHeaders[i].src;
        hdr_names[i] = kHeaders[i].name;
    }
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, source.c_str(), "aether_plan.cu", kNumHeaders, hdr_src, hdr_names) != NVRTC_SUCCESS)
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
    const uint64_t h = cache_key(source, arch, tag, nvrtc_major, nvrtc_minor, -1, nullptr);

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
