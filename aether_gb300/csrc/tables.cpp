// tables.cpp -- the versioned function tables of include/aether_gb300.h.
//
// aether_memory_v1 keeps the layout of the reference seam table
// (dsc/src/seam.h:22-53), so a loader written for that seam binds this
// library unchanged; aether_gb300_v1 adds the fused-expression entry points.

#include "aether_gb300.h"

#include <cuda_runtime.h>

#include <string>

int ag_internal_fail(const char* message);

#define AG_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

// cuFFT is outside the fused-expression path: the seam's optional-missing status.
int fft_plan_missing(int, int, int, int, int, int, const int64_t*, int, const int32_t*, void*, void** plan) {
    if (plan) *plan = nullptr;
    ag_internal_fail("fft_plan: batched FFT is not part of this engine (the fused expression path); "
                     "use the reference's cuFFT plugin");
    return AETHER_MISSING;
}
int fft_exec_missing(void*, const void*, void*, void*) {
    ag_internal_fail("fft_exec: batched FFT is not part of this engine");
    return AETHER_MISSING;
}
void fft_destroy_missing(void*) {}

const AetherMemoryV1 kMemory = {
    AETHER_MEMORY_ABI,   aether_probe,       aether_runtime_version, aether_current_device, aether_last_error,
    aether_chunk_alloc,  aether_chunk_release, aether_drain,         aether_fill,           aether_copy,
    aether_stream_wait,  aether_stream_sync, aether_pointer_device,  fft_plan_missing,      fft_exec_missing,
    fft_destroy_missing,
};

const AetherGB300V1 kGB300 = {
    AETHER_GB300_ABI,
    &kMemory,
    aether_stream_create,
    aether_stream_destroy,
    aether_plan_create,
    aether_plan_info,
    aether_plan_workspace_size,
    aether_plan_launch,
    aether_plan_source,
    aether_plan_release,
    aether_plan_launch_noalloc,
    aether_plan_launch_many,
    aether_batch_create,
    aether_batch_set_items,
    aether_batch_launch,
    aether_batch_capture,
    aether_batch_replay,
    aether_batch_info,
    aether_batch_release,
    aether_serve_open,
    aether_serve_submit,
    aether_serve_feed,
    aether_serve_status,
    aether_serve_wait,
    aether_serve_release,
    aether_serve_stats,
    aether_serve_close,
    aether_runtime_eval,
    aether_rtc_header_count,
    aether_rtc_header,
    aether_rtc_digest,
    aether_plan_generate,
    aether_nvrtc_check,
    aether_plan_cache_key,
    aether_rtc_compile,
};

}  // namespace

AG_EXPORT const AetherMemoryV1* aether_memory_v1(void) { return &kMemory; }
AG_EXPORT const AetherGB300V1* aether_gb300_v1(void) { return &kGB300; }
