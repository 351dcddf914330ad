// host_shim.h -- host spellings of the CUDA intrinsics that
// include/aether/gb300/ag_emu64.cuh uses, so the double-float algorithms
// can be compiled as host C++ and checked against long double. Test
// infrastructure only (compiled with -ffp-contract=off: every _rn operation
// rounds once, as on the device).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#define __device__
#define __forceinline__ inline
#define __align__(n) alignas(n)

typedef unsigned int ag_u32;
typedef unsigned long long ag_u64;
typedef long long ag_i64;

inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double __dadd_rn(double a, double b) { return a + b; }
inline float __uint2float_rn(unsigned u) { return (float)u; }
inline float __double2float_rn(double d) { return (float)d; }
inline float __int_as_float(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}
inline int __float_as_int(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}
inline int __double2hiint(double d) {
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return (int)(u >> 32);
}
inline int __double2loint(double d) {
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return (int)(uint32_t)u;
}
inline unsigned __funnelshift_l(unsigned lo, unsigned hi, unsigned shift) {
    const unsigned long long w = ((unsigned long long)hi << 32) | lo;
    return (unsigned)((w << (shift & 31u)) >> 32);
}
inline double __hiloint2double(int hi, int lo) {
    uint64_t u = ((uint64_t)(uint32_t)hi << 32) | (uint32_t)lo;
    double d;
    std::memcpy(&d, &u, 8);
    return d;
}
template <class T>
inline T __ldg(const T* p) { return *p; }
#include <math.h>
using std::isfinite;

namespace ag {
struct q4 {
    ag_u32 x, y, z, w;
};
inline q4 philox_block(ag_u64 seed, ag_u32 g, ag_u32 c) {
    q4 r = {c, 0u, g, 0u};
    ag_u32 kx = (ag_u32)seed, ky = (ag_u32)(seed >> 32);
    for (int i = 0; i < 10; ++i) {
        if (i) {
            kx += 0x9E3779B9u;
            ky += 0xBB67AE85u;
        }
        const ag_u64 p0 = (ag_u64)0xD2511F53u * r.x, p1 = (ag_u64)0xCD9E8D57u * r.z;
        r = q4{(ag_u32)(p1 >> 32) ^ r.y ^ kx, (ag_u32)p1, (ag_u32)(p0 >> 32) ^ r.w ^ ky, (ag_u32)p0};
    }
    return r;
}
#define AG_HOST_NATIVE(N) inline double f_##N(double x) { return std::N(x); }
AG_HOST_NATIVE(expm1) AG_HOST_NATIVE(exp2) AG_HOST_NATIVE(log2) AG_HOST_NATIVE(log10) AG_HOST_NATIVE(tan)
AG_HOST_NATIVE(asin) AG_HOST_NATIVE(acos) AG_HOST_NATIVE(atan) AG_HOST_NATIVE(tanh) AG_HOST_NATIVE(sinh)
AG_HOST_NATIVE(cosh) AG_HOST_NATIVE(floor) AG_HOST_NATIVE(ceil) AG_HOST_NATIVE(trunc) AG_HOST_NATIVE(cbrt)
AG_HOST_NATIVE(erf)
#undef AG_HOST_NATIVE
inline double f_pow(double a, double b) { return std::pow(a, b); }
inline double f_atan2(double a, double b) { return std::atan2(a, b); }
inline double f_hypot(double a, double b) { return std::hypot(a, b); }
}  // namespace ag
inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz((unsigned)x); }
inline int __clzll(long long x) { return x == 0 ? 64 : __builtin_clzll((unsigned long long)x); }
