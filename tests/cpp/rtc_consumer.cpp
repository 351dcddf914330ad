// What a code generator does with the NVRTC payload: emit a kernel against
// aether/device.h (the reference's consumer spelling), compile it with
// aether_rtc_compile, load the CUBIN with the CUDA driver API and launch it
// on arrays owned by aether::Array, with typed views as kernel parameters.
// The kernel draws a, b per sample from Philox leaves and writes
// d = a + b*c-style terms; the host writes a, b, d (capacity layout) to
// argv[1] for the oracle comparison. Prints "rtc consumer ok".
//
// usage: rtc_consumer <out.bin> <n> <libcu++ include dir> [extra NVRTC option]
#include <aether/aether.h>
#include <cuda.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace {

const char* kSource = R"(
#include "aether/device.h"
using V3 = aether::View<double, aether::extents<3, aether::dyn>, aether::layout_stride>;
extern "C" __global__ void generated(V3 a, V3 b, V3 d, aether::random::Generator g) {
    const aether::SampleIndex i = aether::SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
    if (i.global() >= d.samples()) return;
    a[i] = g.substream(0).uniform<double, 3>(-1.0, 1.0);
    b[i] = g.substream(1).uniform<double, 3>(-1.0, 1.0);
    d[i] = a.cross(b) + a * b;
}
)";

bool ok(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::printf("%s: %s\n", what, s ? s : "?");
    return false;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    const std::size_t n = std::strtoull(argv[2], nullptr, 10);
    aether::Array<double, 3> a(n), b(n), d(n);   // initialises the device's primary context

    std::vector<std::string> opts = {std::string("--include-path=") + argv[3], "--fmad=false"};
    if (argc > 4) opts.push_back(argv[4]);
    std::vector<const char*> copts;
    for (const std::string& o : opts) copts.push_back(o.c_str());
    std::size_t len = 0;
    if (aether_rtc_compile(kSource, "sm_103a", copts.data(), int(copts.size()), nullptr, 0, &len) != AETHER_OK) {
        std::printf("rtc_compile: %s\n", aether_last_error());
        return 1;
    }
    std::vector<char> cubin(len);
    if (aether_rtc_compile(kSource, "sm_103a", copts.data(), int(copts.size()), cubin.data(), len, &len) != AETHER_OK)
        return 1;

    if (!ok(cuInit(0), "cuInit")) return 1;
    CUdevice dev;
    CUcontext ctx;
    if (!ok(cuDeviceGet(&dev, 0), "cuDeviceGet") || !ok(cuDevicePrimaryCtxRetain(&ctx, dev), "retain") ||
        !ok(cuCtxSetCurrent(ctx), "cuCtxSetCurrent"))
        return 1;
    CUmodule mod;
    CUfunction fn;
    if (!ok(cuModuleLoadData(&mod, cubin.data()), "cuModuleLoadData") ||
        !ok(cuModuleGetFunction(&fn, mod, "generated"), "cuModuleGetFunction"))
        return 1;
    auto va = a.deviceView();
    auto vb = b.deviceView();
    auto vd = d.deviceView();
    aether::random::Generator g(42);
    void* params[] = {&va, &vb, &vd, &g};
    const auto cfg = aether::cuda::launchConfig(n, 256);
    if (!ok(cuLaunchKernel(fn, unsigned(cfg.blocks), 1, 1, unsigned(cfg.threads), 1, 1, 0, nullptr, params, nullptr),
            "cuLaunchKernel") ||
        !ok(cuCtxSynchronize(), "cuCtxSynchronize"))
        return 1;
    cuModuleUnload(mod);
    std::FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    for (auto* arr : {&a, &b, &d}) {
        arr->download();
        std::fwrite(arr->hostView().data(), sizeof(double), 3 * arr->capacity(), f);
    }
    std::fclose(f);
    cuDevicePrimaryCtxRelease(dev);
    std::printf("rtc consumer ok\n");
    return 0;
}
