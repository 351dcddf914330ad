// aether/macros.h -- execution-space qualifiers of the consumer API.
//
// The spelling of the reference's qualifier macros (aether/macros.h:118-183):
// code written against aether marks per-sample functions AETHER_DEVICEHOST()
// and kernels AETHER_KERNEL(), and compiles either with nvcc (a .cu consumer
// that launches kernels) or with a host C++ compiler (a .cpp consumer that
// allocates, fills and assigns whole views through the engine's fused plans).
//
//   nvcc, device pass   AETHER_DEVICEHOST() = __device__
//   nvcc, host pass     AETHER_DEVICEHOST() = __host__, AETHER_KERNEL() = __global__
//   host compiler       every qualifier is empty and AETHER_KERNEL is left
//                       undefined, so a kernel in a host translation unit is a
//                       compile error instead of a host function.
#pragma once

#if defined(__CUDACC__)
#define AETHER_DEVICE_COMPILER 1
#else
#define AETHER_DEVICE_COMPILER 0
#endif

#if AETHER_DEVICE_COMPILER
#define AETHER_DEVICE(...) __device__
#define AETHER_HOST(...) __host__
#define AETHER_DEVICEANDHOST(...) __device__ __host__
#define AETHER_NOINLINE(...) __noinline__
#define AETHER_KERNEL(...) __global__
#define AETHER_GRID_CONSTANT(...) const __grid_constant__
#if defined(__CUDA_ARCH__)
#define AETHER_DEVICEHOST(...) __device__
#define AETHER_SHARED(...) __shared__
#define AETHER_DEVICE_COMPILE
#else
#define AETHER_DEVICEHOST(...) __host__
#define AETHER_SHARED(...)
#endif
#else
#define AETHER_DEVICE(...)
#define AETHER_HOST(...)
#define AETHER_DEVICEANDHOST(...)
#define AETHER_DEVICEHOST(...)
#define AETHER_SHARED(...)
#define AETHER_GRID_CONSTANT(...) const
#define AETHER_NOINLINE(...) __attribute__((noinline))
#endif

#if defined(__CUDA_ARCH__)
#define AETHER_FORCEINLINE(...) __forceinline__
#else
#define AETHER_FORCEINLINE(...) inline
#endif

// One unrolled loop over the components of a sample.
#if defined(__CUDA_ARCH__)
#define AETHER_UNROLL _Pragma("unroll")
#else
#define AETHER_UNROLL
#endif
