// aether/aether.h -- the consumer API of the GB300 engine (umbrella header).
//
// The reference's umbrella (aether/aether.h:176-262) for the fused-expression
// path, in two uses of one set of types:
//
// 1. Per-sample code in a consumer's own kernel (a .cu file compiled by nvcc
//    with -I include): typed views, SampleIndex, expressions, Items and the
//    math facade evaluate one sample per thread, the reference's model.
//
//      AETHER_KERNEL() void k(aether::VecView<double, 3> a, aether::VecView<double, 3> d) {
//          const aether::SampleIndex i = aether::SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
//          if (i.global() >= a.samples()) return;
//          d[i] = a + aether::cwiseSin(a) * aether::cwiseExp((a * a) * -1.0);
//      }
//
// 2. Whole-view assignment from host code (any C++17 compiler, no CUDA
//    compiler needed): the same expression assigned to a device view on the
//    host becomes one sm_103a kernel that the library generates, compiles and
//    caches (aether/eval.h).
//
//      aether::Array<double, 3> a(n), b(n), c(n), d(n);
//      aether::random::Generator g(42);
//      a.deviceView() = g.substream(0).uniform<double, 3>(-1.0, 1.0);
//      d.deviceView() = a.deviceView() + b.deviceView() * c.deviceView();
//      d.download();
#pragma once

#include "aether/macros.h"
#include "aether/layout.h"
#include "aether/math.h"
#include "aether/expression.h"
#include "aether/nodes.h"
#include "aether/geometry.h"
#include "aether/view.h"
#include "aether/item.h"
#include "aether/bundle.h"
#include "aether/random.h"
#include "aether/array.h"
#include "aether/eval.h"
#include "aether/accum.h"
#include "aether/accum_run.h"
#include "aether/accum_atomic.h"
#include "aether/rt.h"
#include "aether/batch.h"
#include "aether/device_flag.h"
#include "aether/launch.h"
#include "aether/partition.h"
#include "aether/runtime.h"
#include "aether/reshape.h"
#include "aether/view_copy.h"
#include "aether/chunk.h"
#include "aether/append_counter.h"
#include "aether/dlpack.h"
#include "aether/buffer.h"

#include <cstdint>

// Index aliases and version queries of the reference's umbrella
// (aether/typedefs.h, aether/version.h).
#ifndef AETHER_INDEX_T
#define AETHER_INDEX_T std::uint32_t
#endif
#ifndef AETHER_VERSION_STRING
#define AETHER_VERSION_STRING "unknown"
#endif
#ifndef AETHER_GIT_REVISION
#define AETHER_GIT_REVISION "unknown"
#endif

namespace aether {
inline constexpr int version_major = 0;
using index_base_t = AETHER_INDEX_T;
using idx_t = index_base_t;
using dims_t = index_base_t;
AETHER_DEVICEANDHOST() constexpr const char* version() { return AETHER_VERSION_STRING; }
AETHER_DEVICEANDHOST() constexpr const char* gitRevision() { return AETHER_GIT_REVISION; }
/** The consumer source API's tag, the reference's. */
AETHER_DEVICEANDHOST() constexpr const char* abi() { return "aether-abi-1"; }
}  // namespace aether
