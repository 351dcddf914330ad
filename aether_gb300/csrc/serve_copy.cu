// serve_copy.cu -- operand uploads of the serving loop as one kernel.
//
// A launch slot may need dozens of operands copied in from host memory; one
// cudaMemcpyAsync each costs a copy-engine submission apiece, which for the
// ~1 MB operands of the mixed workload dominates the copy itself. When every
// source is pinned host memory mapped into the device's address space (the
// caller checks with cudaPointerGetAttributes) the SMs read it directly over
// the chip-to-chip link instead: one launch copies every segment of the slot,
// 16 bytes per access, several accesses in flight per thread.

#include <cuda_runtime.h>

#include <cstdint>

#include "serve_copy.h"

namespace {

constexpr int kThreads = 256;
constexpr int kUnroll = 4;

__global__ void __launch_bounds__(kThreads) gather_segments(AgCopyBatch b) {
    const uint64_t stride = uint64_t(gridDim.x) * kThreads;
    for (int s = 0; s < b.n; ++s) {
        const AgCopySegment seg = b.seg[s];
        const int4* __restrict__ src = reinterpret_cast<const int4*>(seg.src);
        int4* __restrict__ dst = reinterpret_cast<int4*>(seg.dst);
        const uint64_t units = seg.bytes / 16;
        uint64_t u = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
        for (; u + (kUnroll - 1) * stride < units; u += kUnroll * stride) {
            int4 v[kUnroll];
#pragma unroll
            for (int k = 0; k < kUnroll; ++k) v[k] = src[u + k * stride];
#pragma unroll
            for (int k = 0; k < kUnroll; ++k) dst[u + k * stride] = v[k];
        }
        for (; u < units; u += stride) dst[u] = src[u];
        // the last bytes % 16 bytes
        const uint64_t tail = seg.bytes - units * 16;
        if (blockIdx.x == 0 && threadIdx.x < tail)
            static_cast<unsigned char*>(seg.dst)[units * 16 + threadIdx.x] =
                static_cast<const unsigned char*>(seg.src)[units * 16 + threadIdx.x];
    }
}

}  // namespace

cudaError_t ag_gather_copy(const AgCopyBatch& b, int sms, cudaStream_t s) {
    if (b.n <= 0) return cudaSuccess;
    uint64_t total = 0;
    for (int i = 0; i < b.n; ++i) total += b.seg[i].bytes;
    const uint64_t want = (total / 16 + kThreads * kUnroll - 1) / (kThreads * kUnroll);
    const uint64_t cap = uint64_t(sms > 0 ? sms : 1) * 4;
    const unsigned grid = unsigned(want < 1 ? 1 : (want < cap ? want : cap));
    gather_segments<<<grid, kThreads, 0, s>>>(b);
    return cudaGetLastError();
}
