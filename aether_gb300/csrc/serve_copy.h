// serve_copy.h -- the serving loop's gather-copy kernel (serve_copy.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

struct AgCopySegment {
    const void* src;   // device-accessible (mapped pinned host memory or device memory), 16-byte aligned
    void* dst;         // device memory, 16-byte aligned
    uint64_t bytes;
};

constexpr int kAgCopyMaxSegments = 128;

// Passed by value as the kernel's parameter (128 * 24 + 8 bytes).
struct AgCopyBatch {
    int n;
    AgCopySegment seg[kAgCopyMaxSegments];
};

// Copy every segment of `b` in one launch on `s`, with a grid sized for `sms`
// SMs. Returns the launch status.
cudaError_t ag_gather_copy(const AgCopyBatch& b, int sms, cudaStream_t s);
