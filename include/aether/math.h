// aether/math.h -- the scalar math facade, host and device.
//
// aether::math (math/math.h:82-287) names one function per operation for
// per-sample code. As in the reference's dispatch (math/detail/
// MathDispatch.h:54-112) the host routes to std:: and the device to CUDA's
// functions, with two choices of this engine:
//   * rsqrt is 1/sqrt(x) with both steps correctly rounded on both sides (the
//     host spelling of math/root.h:63-76), so a device result equals the
//     reference's CPU result bit for bit;
//   * a consumer translation unit compiled with AETHER_GB300_EMULATED_FP64
//     defined evaluates the double sqrt, rsqrt, exp, log, log1p, sin and cos
//     in double-float arithmetic on the FP32/INT pipes (aether/gb300/
//     ag_emu64.cuh, the lowering of the engine's emulated plans): about 2^-46
//     relative per function instead of 2^-53, far faster on GB300's FP64
//     pipe. Arguments outside that arithmetic's range (|x| outside [2^-50,
//     2^60], exp arguments outside (-70, 87), trig arguments beyond 2^24,
//     special values) and results that would not reassemble exactly take
//     CUDA's FP64 function instead, so range and special values keep FP64
//     semantics;
//   * one compiled with AETHER_GB300_FP64_GRADE defined evaluates the same
//     functions in triple-float arithmetic on the FP32/INT pipes (aether/
//     gb300/ag_tf64.cuh and ag_tf64_trig.cuh, the lowering of the engine's
//     FP64-grade plans): within a small fraction of an ulp before the one
//     rounding to double, the FP64 contract, with CUDA's FP64 function for
//     |x| outside [2^-40, 2^60], exp arguments outside (-55, 87), trig
//     arguments beyond 2^10 or near nonzero multiples of pi/2, and special
//     values. The two macros exclude each other.
// The set is the reference's (math/math.h:20-32): the exponential, logarithmic,
// root, trigonometric, hyperbolic and inverse functions, erf and erfc, the
// rounding family (round half away from zero, rint half to even), fmod, fdim,
// numpy's floored remainder, copysign, min/max/fmin/fmax, sign, clip, fma,
// sincos and the classification predicates.
// Every function is usable from device and host code.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <cmath>
#endif

#include "aether/macros.h"

#if defined(AETHER_GB300_EMULATED_FP64) && defined(AETHER_GB300_FP64_GRADE)
#error "aether/math.h: define at most one of AETHER_GB300_EMULATED_FP64 and AETHER_GB300_FP64_GRADE"
#endif
#if defined(__CUDACC__) && defined(AETHER_GB300_EMULATED_FP64)
#include "aether/gb300/ag_device.cuh"
#include "aether/gb300/ag_emu64.cuh"
#endif
// ag_tf64_trig.cuh brings ag_tf64.cuh and ag_emu64.cuh by their bare names
// (one copy each under NVRTC, whose payload also names them by these paths)
#if defined(__CUDACC__) && defined(AETHER_GB300_FP64_GRADE)
#include "aether/gb300/ag_device.cuh"
#include "aether/gb300/ag_tf64_trig.cuh"
#endif

namespace aether {
namespace math {

#if defined(__CUDA_ARCH__) && defined(AETHER_GB300_EMULATED_FP64)
namespace emu {
// One double-float evaluation of f at x, or CUDA's FP64 function where the
// double-float path cannot answer.
#define AETHER_GB300_EMU1(NAME, BODY, NATIVE)                                  \
    __device__ inline double NAME(double x) {                                  \
        bool ok = true;                                                        \
        const ::ag::e64::df v = ::ag::e64::from_double_ck(x, ok);              \
        const ::ag::e64::df r = BODY;                                          \
        const double y = ::ag::e64::to_double(r);                              \
        return (ok && ::ag::e64::out_ok(r) && y == y) ? y : NATIVE(x);         \
    }
__device__ inline double native_rsqrt(double x) { return __ddiv_rn(1.0, __dsqrt_rn(x)); }
AETHER_GB300_EMU1(sqrt, ::ag::e64::sqrt_(v), __dsqrt_rn)
AETHER_GB300_EMU1(rsqrt, ::ag::e64::rsqrt_(v), native_rsqrt)
AETHER_GB300_EMU1(exp, ::ag::e64::exp_(v, ok), ::exp)
AETHER_GB300_EMU1(log, ::ag::e64::log_(v), ::log)
AETHER_GB300_EMU1(log1p, ::ag::e64::log1p_(v), ::log1p)
AETHER_GB300_EMU1(sin, ::ag::e64::sin_(v, ok), ::sin)
AETHER_GB300_EMU1(cos, ::ag::e64::cos_(v, ok), ::cos)
#undef AETHER_GB300_EMU1
}  // namespace emu
#define AETHER_GB300_D(EMU, NATIVE) EMU
#elif defined(__CUDA_ARCH__) && defined(AETHER_GB300_FP64_GRADE)
namespace emu {
// One triple-float evaluation of f at x, or CUDA's FP64 function where the
// triple-float path cannot answer.
#define AETHER_GB300_TF1(NAME, BODY, NATIVE)                                   \
    __device__ inline double NAME(double x) {                                  \
        bool ok = true;                                                        \
        const ::ag::t64::tf v = ::ag::t64::from_double_ck(x, ok);              \
        const ::ag::t64::tf r = BODY;                                          \
        const double y = ::ag::t64::to_double(r);                              \
        return (ok && ::ag::t64::out_ok(r) && y == y) ? y : NATIVE(x);         \
    }
__device__ inline double native_rsqrt(double x) { return __ddiv_rn(1.0, __dsqrt_rn(x)); }
AETHER_GB300_TF1(sqrt, ::ag::t64::sqrt_(v), __dsqrt_rn)
AETHER_GB300_TF1(rsqrt, ::ag::t64::rsqrt_(v), native_rsqrt)
AETHER_GB300_TF1(exp, ::ag::t64::exp_(v, ok), ::exp)
AETHER_GB300_TF1(log, ::ag::t64::log_(v), ::log)
AETHER_GB300_TF1(log1p, ::ag::t64::log1p_(v), ::log1p)
AETHER_GB300_TF1(sin, ::ag::t64::sin_(v, ok), ::sin)
AETHER_GB300_TF1(cos, ::ag::t64::cos_(v, ok), ::cos)
#undef AETHER_GB300_TF1
}  // namespace emu
#define AETHER_GB300_D(EMU, NATIVE) EMU
#else
#define AETHER_GB300_D(EMU, NATIVE) NATIVE
#endif

// -- one-argument functions -------------------------------------------------
#if defined(__CUDA_ARCH__)
#define AETHER_MATH1(NAME, DDEV, FDEV, HOST)                                                \
    AETHER_DEVICEANDHOST() inline double NAME(double x) { return DDEV(x); }                 \
    AETHER_DEVICEANDHOST() inline float NAME(float x) { return FDEV(x); }
#else
#define AETHER_MATH1(NAME, DDEV, FDEV, HOST)                                                \
    AETHER_DEVICEANDHOST() inline double NAME(double x) { return HOST(x); }                 \
    AETHER_DEVICEANDHOST() inline float NAME(float x) { return HOST(x); }
#endif

#if defined(__CUDA_ARCH__)
namespace dev {
__device__ inline double rsqrt(double x) { return __ddiv_rn(1.0, __dsqrt_rn(x)); }
__device__ inline float rsqrt(float x) { return __fdiv_rn(1.0f, __fsqrt_rn(x)); }
__device__ inline double sqrt(double x) { return __dsqrt_rn(x); }
__device__ inline float sqrt(float x) { return __fsqrt_rn(x); }
}  // namespace dev
#endif
#if !defined(__CUDACC_RTC__)
namespace host {
template <class T>
inline T rsqrt(T x) { return T(1) / std::sqrt(x); }
}  // namespace host
#endif

AETHER_MATH1(sqrt, AETHER_GB300_D(emu::sqrt, dev::sqrt), dev::sqrt, std::sqrt)
AETHER_MATH1(rsqrt, AETHER_GB300_D(emu::rsqrt, dev::rsqrt), dev::rsqrt, host::rsqrt)
AETHER_MATH1(exp, AETHER_GB300_D(emu::exp, ::exp), ::expf, std::exp)
AETHER_MATH1(log, AETHER_GB300_D(emu::log, ::log), ::logf, std::log)
AETHER_MATH1(log1p, AETHER_GB300_D(emu::log1p, ::log1p), ::log1pf, std::log1p)
AETHER_MATH1(sin, AETHER_GB300_D(emu::sin, ::sin), ::sinf, std::sin)
AETHER_MATH1(cos, AETHER_GB300_D(emu::cos, ::cos), ::cosf, std::cos)
AETHER_MATH1(cbrt, ::cbrt, ::cbrtf, std::cbrt)
AETHER_MATH1(exp2, ::exp2, ::exp2f, std::exp2)
AETHER_MATH1(expm1, ::expm1, ::expm1f, std::expm1)
AETHER_MATH1(log2, ::log2, ::log2f, std::log2)
AETHER_MATH1(log10, ::log10, ::log10f, std::log10)
AETHER_MATH1(tan, ::tan, ::tanf, std::tan)
AETHER_MATH1(asin, ::asin, ::asinf, std::asin)
AETHER_MATH1(acos, ::acos, ::acosf, std::acos)
AETHER_MATH1(atan, ::atan, ::atanf, std::atan)
AETHER_MATH1(sinh, ::sinh, ::sinhf, std::sinh)
AETHER_MATH1(cosh, ::cosh, ::coshf, std::cosh)
AETHER_MATH1(tanh, ::tanh, ::tanhf, std::tanh)
AETHER_MATH1(erf, ::erf, ::erff, std::erf)
AETHER_MATH1(abs, ::fabs, ::fabsf, std::fabs)
AETHER_MATH1(floor, ::floor, ::floorf, std::floor)
AETHER_MATH1(ceil, ::ceil, ::ceilf, std::ceil)
AETHER_MATH1(trunc, ::trunc, ::truncf, std::trunc)
AETHER_MATH1(round, ::round, ::roundf, std::round)   // half away from zero
AETHER_MATH1(rint, ::rint, ::rintf, std::rint)       // half to even
AETHER_MATH1(asinh, ::asinh, ::asinhf, std::asinh)
AETHER_MATH1(acosh, ::acosh, ::acoshf, std::acosh)
AETHER_MATH1(atanh, ::atanh, ::atanhf, std::atanh)
AETHER_MATH1(erfc, ::erfc, ::erfcf, std::erfc)
#if !defined(__CUDACC_RTC__)
namespace host {
// 10^x: glibc's exp10 where the C library has one, else pow(10, x)
template <class T>
inline T exp10(T x) {
#if defined(__GLIBC__)
    return ::exp10(x);
#else
    return std::pow(T(10), x);
#endif
}
}  // namespace host
#endif
AETHER_MATH1(exp10, ::exp10, ::exp10f, host::exp10)
#undef AETHER_MATH1
#undef AETHER_GB300_D

// -- two- and three-argument functions ---------------------------------------
#if defined(__CUDA_ARCH__)
#define AETHER_MATH2(NAME, DDEV, FDEV, HOST)                                                       \
    AETHER_DEVICEANDHOST() inline double NAME(double a, double b) { return DDEV(a, b); }          \
    AETHER_DEVICEANDHOST() inline float NAME(float a, float b) { return FDEV(a, b); }
#else
#define AETHER_MATH2(NAME, DDEV, FDEV, HOST)                                                       \
    AETHER_DEVICEANDHOST() inline double NAME(double a, double b) { return HOST(a, b); }          \
    AETHER_DEVICEANDHOST() inline float NAME(float a, float b) { return HOST(a, b); }
#endif
AETHER_MATH2(pow, ::pow, ::powf, std::pow)
AETHER_MATH2(atan2, ::atan2, ::atan2f, std::atan2)
AETHER_MATH2(hypot, ::hypot, ::hypotf, std::hypot)
AETHER_MATH2(min, ::fmin, ::fminf, std::fmin)
AETHER_MATH2(max, ::fmax, ::fmaxf, std::fmax)
AETHER_MATH2(fmin, ::fmin, ::fminf, std::fmin)
AETHER_MATH2(fmax, ::fmax, ::fmaxf, std::fmax)
AETHER_MATH2(fmod, ::fmod, ::fmodf, std::fmod)        // sign of the dividend
AETHER_MATH2(fdim, ::fdim, ::fdimf, std::fdim)
AETHER_MATH2(copysign, ::copysign, ::copysignf, std::copysign)
#undef AETHER_MATH2

// -- sign, clip, remainder and the classification predicates ----------------
// The reference's semantics (math/math.h:155-215, math/round.h:94-115): sign
// is 0 for either zero and for NaN; clip lets NaN through and clamps the rest
// to [lo, hi]; remainder is the floored remainder of numpy (the result takes
// the divisor's sign, an exact zero takes it too), not C's IEEE remainder.
template <class T>
AETHER_DEVICEANDHOST() inline T clip(T x, T lo, T hi) {
    const bool nan = x != x;
    const T t = (nan || x >= lo) ? x : lo;
    return (nan || t <= hi) ? t : hi;
}
template <class T>
AETHER_DEVICEANDHOST() inline T remainder(T a, T b) {
    T m = fmod(a, b);
    if (m == T(0)) return copysign(T(0), b);
    return ((m < T(0)) != (b < T(0))) ? m + b : m;
}


AETHER_DEVICEANDHOST() inline double fma(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
AETHER_DEVICEANDHOST() inline float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

template <class T>
AETHER_DEVICEANDHOST() inline void sincos(T x, T* s, T* c) {
    *s = math::sin(x);
    *c = math::cos(x);
}

AETHER_DEVICEANDHOST() inline bool isfinite(double x) {
#if defined(__CUDA_ARCH__)
    return ::isfinite(x);
#else
    return std::isfinite(x);
#endif
}
AETHER_DEVICEANDHOST() inline bool isfinite(float x) {
#if defined(__CUDA_ARCH__)
    return ::isfinite(x);
#else
    return std::isfinite(x);
#endif
}
#if defined(__CUDA_ARCH__)
#define AETHER_MATH_PRED(NAME)                                                      \
    AETHER_DEVICEANDHOST() inline bool NAME(double x) { return ::NAME(x); }          \
    AETHER_DEVICEANDHOST() inline bool NAME(float x) { return ::NAME(x); }
#else
#define AETHER_MATH_PRED(NAME)                                                      \
    AETHER_DEVICEANDHOST() inline bool NAME(double x) { return std::NAME(x); }       \
    AETHER_DEVICEANDHOST() inline bool NAME(float x) { return std::NAME(x); }
#endif
AETHER_MATH_PRED(isnan)
AETHER_MATH_PRED(isinf)
#undef AETHER_MATH_PRED

/** -1, 0 or +1 (the sign of math/round.h's sign(), NaN -> 0). */
template <class T>
AETHER_DEVICEANDHOST() constexpr T sign(T x) {
    return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0));
}

}  // namespace math
}  // namespace aether
