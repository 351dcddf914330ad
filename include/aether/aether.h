// aether/aether.h -- the C++ front end of the GB300 engine (umbrella header).
//
// The consumer surface of the reference's umbrella (aether/aether.h:176-262)
// for the fused-assignment path: Array<T, Es...> with host and device views,
// lazy expressions assigned in one statement, aether::math, aether::random.
// Host code compiles with any C++17 compiler and links libaether_gb300.so;
// no CUDA compiler is involved on the consumer side: every assignment becomes
// one sm_103a kernel generated, compiled and cached by the library.
//
//   #include <aether/aether.h>
//   aether::Array<double, 3> a(n), b(n), c(n), d(n);
//   aether::random::Generator g(42);
//   a.deviceView() = g.substream(0).uniform<double, 3>(-1.0, 1.0);
//   ...
//   d.deviceView() = a.deviceView() + b.deviceView() * c.deviceView()
//                    + aether::cwiseSin(a.deviceView()) * aether::cwiseExp((c.deviceView() * c.deviceView()) * -1.0);
//   d.download();
#pragma once

#include "aether/accum.h"
#include "aether/array.h"
#include "aether/batch.h"
#include "aether/device_flag.h"
#include "aether/eval.h"
#include "aether/expr.h"
#include "aether/math.h"
#include "aether/partition.h"
#include "aether/random.h"
#include "aether/runtime.h"

namespace aether {
inline constexpr int version_major = 0;
}  // namespace aether
