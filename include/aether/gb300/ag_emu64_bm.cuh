// ag_emu64_bm.cuh -- the Box-Muller draw in double-float (N(mu, sigma) and
// lognormal leaves of plans lowered with math = 1), included by the generated
// kernels of plans that draw normals, after ag_emu64.cuh.
//
// z = sqrt(-2 log u) sin(pi v) (random/detail/Backend.h:209-236, first normal
// only) from the reference's own double uniforms u and v, reproduced exactly
// in integers; log(u) is taken as log(u) for u < 1/2 and as log1p(-(1-u))
// above, with 1-u formed in integers; sin(pi v) is reduced in integers to a
// point of a table of sin and pi cos of pi k/4096 over the whole period and an
// exact remainder.
#pragma once

#include "ag_emu64_bm_tables.cuh"

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define AG_NOINLINE __noinline__
#else
#define AG_NOINLINE __attribute__((noinline))
#endif

namespace ag {
namespace e64 {

// sgn w 2^-54 for 0 < w < 2^54: normalised so the leading bit sits at 2^53,
// the top 24 bits exact and the next 30 rounded once (2^-48 relative); the
// pair is left with |lo| < ulp(hi). sgn is the sign bit (0 or 0x80000000).
__device__ AG_NOINLINE df from_u54_2m54_any(ag_u64 w, ag_u32 sgn) {
    const int lz = __clzll((long long)w) - 10;   // 0 .. 53
    const ag_u64 wn = w << lz;                    // [2^53, 2^54)
    const ag_u32 sc = ((ag_u32)(103 - lz) << 23) | sgn;   // +-2^(-24-lz): 2^30 units of wn, times 2^-54
    const float h = __fmul_rn(__uint2float_rn((ag_u32)(wn >> 30)), __int_as_float(sc));
    const float l = __fmul_rn(__uint2float_rn((ag_u32)wn & 0x3fffffffu), __int_as_float(sc - (30u << 23)));
    return mk(h, l);
}
// The same in 32-bit words when w >= 2^32 (all but 2^-22 of the draws: the
// normalising shift stays below 32), the general form out of line otherwise.
// No integer-to-float conversion unit: the head's float is assembled from
// its bits (the top 24 bits of w << lz are its significand, the shift gives
// its exponent), and the tail is the next 23 bits made exact by the 2^23
// exponent trick (one OR and one subtraction) and scaled; the 7 bits below
// are dropped, 2^-47 of u.
__device__ __forceinline__ df from_u54_2m54(ag_u64 w, ag_u32 sgn) {
    const ag_u32 hi = (ag_u32)(w >> 32), lo = (ag_u32)w;
    if (hi == 0u) return from_u54_2m54_any(w, sgn);
    const int lz = __clz((int)hi) - 10;   // 0 .. 21
    const ag_u32 nh = __funnelshift_l(lo, hi, (unsigned)lz), nl = lo << lz;   // w << lz in [2^53, 2^54)
    const ag_u32 top = __funnelshift_l(nl, nh, 2u);                           // bits 53..30, in [2^23, 2^24)
    // top 2^(30 - 54 - lz): exponent -1 - lz, significand top
    const float h = __int_as_float((int)(((ag_u32)(126 - lz) << 23) | (top & 0x7fffffu) | sgn));
    // bits 29..7 as an exact float, weight 2^(7 - 54 - lz)
    const float r = __fsub_rn(__int_as_float((int)(0x4B000000u | ((nl >> 7) & 0x7fffffu))), 8388608.0f);
    const float l = __fmul_rn(r, __int_as_float((int)(((ag_u32)(80 - lz) << 23) | sgn)));
    return mk(h, l);
}

// sin(pi (k/4096 + t)) from the table entry (S, pi C) of k and the exact
// remainder |t| <= 2^-13 in half-turns: with r = pi t, S (1 + cm1) + C st,
// st = sin r = r + r^3 (-1/6 + r^2/120) and cm1 = cos r - 1 = r^2 (-1/2 +
// r^2/24). C r = (pi C) t and C r^3 = (pi C) t r^2, so only the float r of the
// small terms needs pi; the leading product is (pi C) t in double-float.
// |S| >= sin(pi/4096) >= |C r| except where S = 0: the sum is led by S.
__device__ __forceinline__ df sin_from_period_table(const f4& sc, df t) {
    const float th = t.hi;
    // r = pi t rounded once (pi's and t's low parts joined by FMA): the
    // quadratic term needs r to float accuracy
    const float rh = __fmaf_rn(AG_PI_HI, th, __fmaf_rn(AG_PI_HI, t.lo, __fmul_rn(AG_PI_LO, th)));
    const float rh2 = __fmul_rn(rh, rh);
    const float cub = __fmul_rn(__fmul_rn(th, rh2), __fmaf_rn(rh2, 8.33333333e-3f, -1.66666667e-1f));
    const float cm1 = __fmul_rn(rh2, __fmaf_rn(rh2, 4.16666667e-2f, -0.5f));
    const df S = mk(sc.x, sc.y), PC = mk(sc.z, sc.w);
    return add_quick(add_quick(S, mul_u(PC, t)), __fmaf_rn(S.hi, cm1, __fmul_rn(PC.hi, cub)));
}

// U: the product is left unnormalised (the draw is only reassembled into a double)
template <bool U = false>
__device__ __forceinline__ df normal_df(ag_u64 seed, ag_u32 g, ag_u32 c) {
    const ag::q4 x = ag::philox_block(seed, g, c);
    // u is the reference's double z 2^-53 + 2^-54 (random/detail/Backend.h
    // uniformDoubleHq): exact below 1/2, rounded to even above it, where it is
    // k 2^-53 with k = z + (z & 1). So u = w 2^-54 with w = 2 z + 1 below 1/2,
    // and 1 - u = w 2^-54 with w = 2^54 - 2 k (even, at most 2^53) above it.
    const ag_u64 z = (ag_u64)x.x ^ ((ag_u64)x.y << 21);
    const bool lower = z < (1ull << 52);
    const ag_u64 w = lower ? 2ull * z + 1ull : (1ull << 54) - 2ull * (z + (z & 1ull));
    // log(u) for u in [2^-54, 1/2) or log1p(-w) for w in [0, 1/2]; w = 0 (u
    // rounded to 1) gives a zero argument to the square root below, whose NaN
    // sends the lane to the native path
    const df L = log_s<false, LOG_SRT>(lower ? 0.0f : 1.0f, from_u54_2m54(w, lower ? 0u : 0x80000000u));
    const df sv = sqrt_pos_(scale(L, -2.0f));   // log u < 0: the argument is positive
    // v is the reference's double zy 2^-52 + 2^-53: exact below 1, rounded to
    // even above it. So v = V 2^-53 with V = 2 zy + 1, or 2 (zy + (zy & 1))
    // for zy >= 2^52, V <= 2^54. In integers: K = round(V / 2^41) in [0, 8192]
    // counts steps of 1/4096 half-turn (the table point pi K/4096), and R = V -
    // 2^41 K (|R| <= 2^40) is the remainder, exact in a double-float: sin(pi v)
    // keeps full relative accuracy next to the zeros of the sine.
    const ag_u64 zy = (ag_u64)x.z ^ ((ag_u64)x.w << 21);
    const ag_u64 V = zy < (1ull << 52) ? 2ull * zy + 1ull : 2ull * (zy + (zy & 1ull));
    const ag_u32 vh = (ag_u32)(V >> 32), vl = (ag_u32)V;
    const ag_u32 K = (vh + 256u) >> 9;   // (V + 2^40) >> 41
    const ag_u32 rh = vh - (K << 9);   // R = rh 2^32 + vl, rh in [-256, 255] as a signed word
    // R = Rh 2^18 + Rl with Rh = floor(R / 2^18) (|Rh| <= 2^22) and 0 <= Rl < 2^18,
    // both made exact floats by exponent tricks (no conversion unit): Rh as
    // (1.5 2^23 + Rh) - 1.5 2^23, Rl as (2^23 + Rl) - 2^23
    const int Rh = (int)((rh << 14) | (vl >> 18));
    const float fh = __fsub_rn(__int_as_float(0x4B400000 + Rh), 12582912.0f);
    const float fl = __fsub_rn(__int_as_float((int)(0x4B000000u | (vl & 0x3ffffu))), 8388608.0f);
    const df t = fast_two_sum(__fmul_rn(fh, p2f(-35)), __fmul_rn(fl, p2f(-53)));
    const df sn = sin_from_period_table(ld4(kSinCosPiPeriod, (int)K), t);
    return U ? mul_u(sv, sn) : mul(sv, sn);
}

}  // namespace e64
}  // namespace ag
