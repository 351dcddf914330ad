// aether/math.h -- the scalar math facade on the host.
//
// aether::math (math/math.h:82-287) names one function per operation for
// per-sample code; on the host the reference routes to std:: (math/detail/
// MathDispatch.h:54-112), with rsqrt as 1/std::sqrt (math/root.h:63-76) and
// log1p/expm1 from <cmath> (math/explog.h:38-81). Device code of this engine
// is generated per expression (the kernels evaluate the elementwise nodes of
// aether/expr.h), so only the host half is declared here.
#pragma once

#include <cmath>

namespace aether {
namespace math {

template <class T> inline T sqrt(T x) { return std::sqrt(x); }
template <class T> inline T rsqrt(T x) { return T(1) / std::sqrt(x); }
template <class T> inline T cbrt(T x) { return std::cbrt(x); }
template <class T> inline T exp(T x) { return std::exp(x); }
template <class T> inline T exp2(T x) { return std::exp2(x); }
template <class T> inline T expm1(T x) { return std::expm1(x); }
template <class T> inline T log(T x) { return std::log(x); }
template <class T> inline T log2(T x) { return std::log2(x); }
template <class T> inline T log10(T x) { return std::log10(x); }
template <class T> inline T log1p(T x) { return std::log1p(x); }
template <class T> inline T sin(T x) { return std::sin(x); }
template <class T> inline T cos(T x) { return std::cos(x); }
template <class T> inline T tan(T x) { return std::tan(x); }
template <class T> inline T asin(T x) { return std::asin(x); }
template <class T> inline T acos(T x) { return std::acos(x); }
template <class T> inline T atan(T x) { return std::atan(x); }
template <class T> inline T atan2(T y, T x) { return std::atan2(y, x); }
template <class T> inline T sinh(T x) { return std::sinh(x); }
template <class T> inline T cosh(T x) { return std::cosh(x); }
template <class T> inline T tanh(T x) { return std::tanh(x); }
template <class T> inline T erf(T x) { return std::erf(x); }
template <class T> inline T abs(T x) { return std::fabs(x); }
template <class T> inline T floor(T x) { return std::floor(x); }
template <class T> inline T ceil(T x) { return std::ceil(x); }
template <class T> inline T trunc(T x) { return std::trunc(x); }
template <class T> inline T pow(T x, T y) { return std::pow(x, y); }
template <class T> inline T hypot(T x, T y) { return std::hypot(x, y); }
template <class T> inline T fma(T a, T b, T c) { return std::fma(a, b, c); }
template <class T> inline T min(T a, T b) { return std::fmin(a, b); }
template <class T> inline T max(T a, T b) { return std::fmax(a, b); }
template <class T> inline void sincos(T x, T* s, T* c) {
    *s = std::sin(x);
    *c = std::cos(x);
}

}  // namespace math
}  // namespace aether
