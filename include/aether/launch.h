// aether/launch.h -- launch helpers for consumer kernels.
//
// aether::cuda::launchConfig and bundleLaunchConfig (backend/cuda/Launch.h:
// 53-74): a 1D grid of `block`-thread blocks covering n samples (one per
// thread), or n samples W per thread. checkLastLaunch (Launch.h:84-88) and
// AETHER_CHECK_CUDA (:98) turn a failed launch or CUDA call into an
// aether::Error worded "<op> failed on <where>, size=0 bytes (<CUDA error>)"
// (err/Error.h:30-87). checkLastLaunch synchronises the device, so it is not
// for use while a stream is being captured; use cudaPeekAtLastError there.
// The checks need the CUDA runtime and exist in nvcc translation units only.
#pragma once

#include <cstddef>
#include <string>

#include "aether/expr.h"

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#endif

namespace aether {
namespace cuda {

struct LaunchConfig {
    int blocks;
    int threads;
};

/** ceil(n / block) blocks of `block` threads. */
inline LaunchConfig launchConfig(std::size_t n, int block = 256) {
    const std::size_t b = static_cast<std::size_t>(block);
    return LaunchConfig{static_cast<int>((n + b - 1) / b), block};
}

/** One thread per W-sample bundle: ceil(ceil(n / W) / block) blocks. */
inline LaunchConfig bundleLaunchConfig(std::size_t n, std::size_t W, int block = 256) {
    return launchConfig((n + W - 1) / W, block);
}

}  // namespace cuda

#if defined(__CUDACC__)
namespace err {
/** Throws aether::Error for a failed CUDA status (err/Error.h:30-87). */
inline void checkCuda(cudaError_t status, const std::string& op, const std::string& where, std::size_t bytes) {
    if (status != cudaSuccess)
        throw Error::memory(op, where, bytes, std::string(cudaGetErrorName(status)) + ": " + cudaGetErrorString(status));
}
}  // namespace err

namespace cuda {
/** The kernel launched just before started and ran to completion. */
inline void checkLastLaunch(const char* name) {
    err::checkCuda(cudaGetLastError(), std::string("checkLastLaunch(") + name + ")", "CUDA[launch]", 0);
    err::checkCuda(cudaDeviceSynchronize(), std::string("checkLastLaunch(") + name + ")", "CUDA[execution]", 0);
}
}  // namespace cuda
#endif

}  // namespace aether

#if defined(__CUDACC__)
#define AETHER_CHECK_CUDA(call) ::aether::err::checkCuda((call), #call, "CUDA", 0)
#endif
