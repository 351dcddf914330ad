// ag_fastdiv.cuh -- division of 32-bit unsigned integers by an invariant
// divisor with one high multiply (Granlund & Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994, Theorem 4.2).
//
// For d >= 1 let l = ceil(log2 d) and m = floor(2^(32+l) / d) + 1; then
// floor(x / d) = floor(m * x / 2^(32+l)) for every x < 2^32. m exceeds 32
// bits, so it is kept as 2^32 + mp and the quotient is formed as
// (x + mulhi(mp, x)) >> l in 64-bit arithmetic. Host and device share this
// code; the host test checks it against the hardware divide.
#pragma once

#ifndef __CUDACC__
#define AG_FD_HD
#else
#define AG_FD_HD __host__ __device__
#endif

#include <stdint.h>

struct AgFastDiv {
    uint32_t d;
    uint32_t mp;
    uint32_t l;
};

inline AG_FD_HD AgFastDiv ag_fastdiv_make(uint32_t d) {
    AgFastDiv f;
    f.d = d;
    uint32_t l = 0;
    while (l < 32 && (uint64_t(1) << l) < uint64_t(d)) ++l;
    f.l = l;
    // mp = floor(2^32 * (2^l - d) / d) + 1
    f.mp = uint32_t(((uint64_t(1) << 32) * ((uint64_t(1) << l) - uint64_t(d))) / uint64_t(d) + 1u);
    return f;
}

inline AG_FD_HD uint32_t ag_fastdiv_div(uint32_t x, const AgFastDiv& f) {
#ifdef __CUDA_ARCH__
    const uint32_t t = __umulhi(f.mp, x);
#else
    const uint32_t t = uint32_t((uint64_t(f.mp) * uint64_t(x)) >> 32);
#endif
    return uint32_t((uint64_t(t) + uint64_t(x)) >> f.l);
}

// x = q * d + r
inline AG_FD_HD void ag_fastdiv_divmod(uint32_t x, const AgFastDiv& f, uint32_t& q, uint32_t& r) {
    q = ag_fastdiv_div(x, f);
    r = x - q * f.d;
}
