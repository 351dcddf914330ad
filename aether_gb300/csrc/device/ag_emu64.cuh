// ag_emu64.cuh -- FP64 math evaluated on the FP32 and integer pipes.
//
// Included by generated kernels lowered with math = 1. On GB300 the FP64 pipe
// issues about 1.6 operations per clock per SM against about 110 FFMA and 59
// IMAD, so an FP64 expression kernel with transcendental nodes is bound by the
// FP64 pipe long before HBM. The functions here keep FP64 inputs and outputs
// but do the bulk of the arithmetic in float/integer form.
#pragma once

namespace ag {
namespace e64 {

// Until a node has an emulated form it falls back to the native one.
using ag::f_abs;
using ag::f_acos;
using ag::f_asin;
using ag::f_atan;
using ag::f_atan2;
using ag::f_cbrt;
using ag::f_ceil;
using ag::f_cos;
using ag::f_cosh;
using ag::f_erf;
using ag::f_exp;
using ag::f_exp2;
using ag::f_expm1;
using ag::f_floor;
using ag::f_hypot;
using ag::f_log;
using ag::f_log10;
using ag::f_log1p;
using ag::f_log2;
using ag::f_max;
using ag::f_min;
using ag::f_neg;
using ag::f_pow;
using ag::f_rsqrt;
using ag::f_sign;
using ag::f_sin;
using ag::f_sinh;
using ag::f_sqrt;
using ag::f_tan;
using ag::f_tanh;
using ag::f_trunc;

}  // namespace e64
}  // namespace ag
