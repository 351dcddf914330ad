// aether/detail/std.h -- the standard-library facilities of the device-side
// headers, for every compiler that builds them.
//
// nvcc and host compilers use the real <cstddef>, <cstdint>, <type_traits>
// and <utility>. NVRTC has no C++ standard library; there the same names come
// from the CUDA toolkit's libcu++ (cuda::std, NVRTC-safe by construction),
// re-exported into ::std, so the headers of aether/device.h compile unchanged
// in a code generator's NVRTC program (compile with
// --include-path=<CUDA>/include/cccl, or <CUDA>/include on toolkits that keep
// libcu++ there).
#pragma once

#if defined(__CUDACC_RTC__)
#include <cuda/std/cstddef>
#include <cuda/std/cstdint>
#include <cuda/std/type_traits>
#include <cuda/std/utility>
namespace std {
using namespace cuda::std;
}
#else
#include <cstddef>
#include <cstdint>
#include <type_traits>
#include <utility>
#endif
