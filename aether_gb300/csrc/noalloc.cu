// noalloc.cu -- launching a sum plan without any device allocation.
//
// A sum plan needs device scratch: a completion counter plus one (hi, comp)
// partial per chunk of samples. aether_plan_launch takes it from the caller
// or allocates it for the plan on first use. Some callers cannot allocate at
// the point where they launch: hosts that run under a fixed device-memory
// budget (a serving loop that admits work by bytes) must not grow it behind
// their back, and latency-critical loops cannot afford an allocation stall.
// For them, aether_plan_launch_noalloc takes the scratch from a fixed array
// compiled into this library instead.
//
// The array is a file-scope static __device__ buffer of AG_NOALLOC_SCRATCH_BYTES
// (1 MiB) that every GPU which loads the library holds until the process
// exits. Its device address is resolved once per device, on the first call
// made with that device current (cudaGetSymbolAddress); a first call on a
// stream that is capturing is refused. The address is kept for the life of the process: after a
// cudaDeviceReset the entry point is not usable, as plans are not. All calls
// share the one array: the counter is cleared at the start of every call, and
// calls whose kernels overlap on the GPU (two streams, or two threads) race
// on it; serialise them.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "aether_gb300.h"

#define AG_NOALLOC_SCRATCH_BYTES (1u << 20)
#define AG_NOALLOC_MAX_DEVICES 64

int ag_internal_fail(const char* message);

static __device__ __align__(256) unsigned char g_noalloc_scratch[AG_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_mu;
void* g_addr[AG_NOALLOC_MAX_DEVICES] = {};

int fail_msg(const std::string& m) { return ag_internal_fail(m.c_str()); }

}  // namespace

extern "C" __attribute__((visibility("default"))) int aether_plan_launch_noalloc(void* plan, const AetherLaunch* args,
                                                                                  void* stream) {
    if (!plan || !args) return fail_msg("plan_launch_noalloc: null argument");
    if (args->workspace) return fail_msg("plan_launch_noalloc: the scratch is the library's own; pass workspace = NULL");
    AetherPlanInfo info;
    if (aether_plan_info(plan, &info) != AETHER_OK) return AETHER_FAIL;
    if (!info.is_sum) return fail_msg("plan_launch_noalloc: only sum plans use scratch; launch this plan with aether_plan_launch");
    uint64_t need = 0;
    if (aether_plan_workspace_size(plan, args->n, &need) != AETHER_OK) return AETHER_FAIL;
    if (need > AG_NOALLOC_SCRATCH_BYTES)
        return fail_msg("plan_launch_noalloc: " + std::to_string(args->n) + " samples need " + std::to_string(need) +
                        " bytes of scratch; the static scratch holds " + std::to_string(AG_NOALLOC_SCRATCH_BYTES) +
                        " bytes (16 + 16 per chunk); split the sum or use aether_plan_launch");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_msg(std::string("plan_launch_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= AG_NOALLOC_MAX_DEVICES) return fail_msg("plan_launch_noalloc: device index out of range");
    void* ptr = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            // resolving the symbol may load the module; never do that inside
            // a caller's capture
            cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
            e = cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &st);
            if (e != cudaSuccess)
                return fail_msg(std::string("plan_launch_noalloc: cudaStreamIsCapturing: ") + cudaGetErrorString(e));
            if (st != cudaStreamCaptureStatusNone)
                return fail_msg("plan_launch_noalloc: the first call on a device must come before any stream "
                                "capture (it resolves the static scratch's address); make one uncaptured call first");
            e = cudaGetSymbolAddress(&g_addr[dev], g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_addr[dev] = nullptr;
                cudaGetLastError();
                return fail_msg(std::string("plan_launch_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            }
        }
        ptr = g_addr[dev];
    }
    AetherLaunch a = *args;
    a.workspace = ptr;
    a.workspace_bytes = AG_NOALLOC_SCRATCH_BYTES;
    // aether_plan_launch with a caller workspace clears the counter with
    // cudaMemsetAsync and launches; it allocates nothing.
    return aether_plan_launch(plan, &a, stream);
}
