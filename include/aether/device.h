// aether/device.h -- the device-safe half of the consumer API.
//
// The reference's NVRTC-parseable umbrella (aether/device.h:1-30): what a code
// generator that compiles its own kernels with NVRTC includes -- macros,
// extents and layouts, SampleIndex, views with `view[i] = expr`, Items, the
// expression nodes, aether::math and the Philox leaves -- without the
// host-only parts (arrays, the engine's whole-view launches, batches,
// serving). The library exports these headers, and the device runtime of
// aether/gb300/ they reach, as its NVRTC payload (aether_rtc_header*), each
// under the include name used here; aether_rtc_compile compiles a source
// against that payload. Under NVRTC the standard facilities come from
// libcu++ (aether/detail/std.h). nvcc and host compilers can include this
// header too.
#pragma once

#include "aether/macros.h"
#include "aether/detail/std.h"
#include "aether/layout.h"
#include "aether/math.h"
#include "aether/expression.h"
#include "aether/nodes.h"
#include "aether/geometry.h"
#include "aether/view.h"
#include "aether/item.h"
#include "aether/bundle.h"
#include "aether/detail/philox.h"
#include "aether/random.h"
