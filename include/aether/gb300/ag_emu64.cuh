// ag_emu64.cuh -- FP64 expression math on the FP32 and integer pipes.
//
// Included by generated kernels lowered with math = 1. On GB300 the FP64 pipe
// issues about 1.6 operations per clock per SM against about 110 FFMA and 59
// IMAD (double <-> float conversions run on the FP64 pipe as well), so an
// FP64 expression kernel with transcendental nodes is bound by that pipe long
// before HBM. Here every double is split into a double-float pair
// (hi + lo, two floats, about 48 significant bits) with integer operations,
// the expression is evaluated in double-float arithmetic, and each output is
// reassembled into a double with one FP64 addition.
//
// Accuracy: relative error about 2^-46 per function (a few tens of double
// ulps in the worst case), against 2^-53 for the native pipe. Samples whose
// inputs leave [2^-50, 2^60] in magnitude, whose products or quotients fall
// below 2^-102 (where the pair's error terms would be subnormal), whose exp
// arguments leave (-70, 87), whose trig arguments reach 2^24, or whose
// outputs are not finite normal values above 2^-90 are recomputed by the
// generated code with native FP64 (the fallback path), so range, special
// values and large-argument reduction keep FP64 semantics.
//
// Methods (all from the published literature, constants computed by
// gen_emu64_tables.py): Knuth two-sum, Dekker fast-two-sum, FMA two-product;
// double-word addition/multiplication of Joldes, Muller & Popescu (2017);
// Newton-Raphson square root and reciprocal square root from a hardware seed;
// table-driven exp (Tang 1989) and log (Tang 1990); Cody-Waite reduction by
// pi/2 with a 1/32-spaced sine/cosine table; Box-Muller from exact integer
// uniforms.
#pragma once

#include "ag_emu64_tables.cuh"

namespace ag {
namespace e64 {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df mk(float h, float l) {
    df r;
    r.hi = h;
    r.lo = l;
    return r;
}

// One 16-byte table entry (the packed (hi, lo, hi, lo) rows of the tables).
struct f4 {
    float x, y, z, w;
};
__device__ __forceinline__ f4 ld4(const float* tab, int row) {
#ifdef __CUDA_ARCH__
    const float4 v = __ldg(reinterpret_cast<const float4*>(tab) + row);
    return f4{v.x, v.y, v.z, v.w};
#else
    const float* p = tab + 4 * row;
    return f4{p[0], p[1], p[2], p[3]};
#endif
}

// ---------------------------------------------------------------------------
// Error-free transformations.
// ---------------------------------------------------------------------------
__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return mk(s, e);
}
// Requires |a| >= |b| or a == 0.
__device__ __forceinline__ df fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return mk(s, e);
}
__device__ __forceinline__ df two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return mk(p, e);
}

// ---------------------------------------------------------------------------
// Double-float arithmetic.
// ---------------------------------------------------------------------------
__device__ __forceinline__ df neg(df x) { return mk(-x.hi, -x.lo); }

// Accurate sum, relative error <= 3u^2 even under cancellation.
__device__ __forceinline__ df add(df x, df y) {
    const df s = two_sum(x.hi, y.hi);
    const df t = two_sum(x.lo, y.lo);
    const float c = __fadd_rn(s.lo, t.hi);
    const df v = fast_two_sum(s.hi, c);
    const float w = __fadd_rn(t.lo, v.lo);
    return fast_two_sum(v.hi, w);
}
__device__ __forceinline__ df sub(df x, df y) { return add(x, neg(y)); }
// Sum of terms that cannot cancel (same sign, or |y| well below |x|).
__device__ __forceinline__ df add_fast(df x, df y) {
    const df s = two_sum(x.hi, y.hi);
    const float v = __fadd_rn(__fadd_rn(x.lo, y.lo), s.lo);
    return fast_two_sum(s.hi, v);
}
// The same sum left unnormalised, for a value whose only reader is the
// reassembly into a double (which rounds hi + lo once either way).
__device__ __forceinline__ df add_fast_u(df x, df y) {
    const df s = two_sum(x.hi, y.hi);
    return mk(s.hi, __fadd_rn(__fadd_rn(x.lo, y.lo), s.lo));
}
__device__ __forceinline__ df add(df x, float y) {
    const df s = two_sum(x.hi, y);
    const float v = __fadd_rn(x.lo, s.lo);
    return fast_two_sum(s.hi, v);
}
__device__ __forceinline__ df mul(df x, df y) {
    const df c = two_prod(x.hi, y.hi);
    const float tl0 = __fmul_rn(x.lo, y.lo);
    const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
    const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
    return fast_two_sum(c.hi, __fadd_rn(c.lo, cl2));
}
__device__ __forceinline__ df mul(df x, float y) {
    const df c = two_prod(x.hi, y);
    return fast_two_sum(c.hi, __fmaf_rn(x.lo, y, c.lo));
}
__device__ __forceinline__ df sqr(df x) {
    const df c = two_prod(x.hi, x.hi);
    return fast_two_sum(c.hi, __fmaf_rn(2.0f * x.hi, x.lo, c.lo));
}
// Products whose only consumer is a sum: the same pair before the final
// Fast2Sum (|lo| up to about one ulp of hi), which every sum below accepts.
__device__ __forceinline__ df mul_u(df x, df y) {
    const df c = two_prod(x.hi, y.hi);
    const float tl0 = __fmul_rn(x.lo, y.lo);
    const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
    const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
    return mk(c.hi, __fadd_rn(c.lo, cl2));
}
__device__ __forceinline__ df mul_u(df x, float y) {
    const df c = two_prod(x.hi, y);
    return mk(c.hi, __fmaf_rn(x.lo, y, c.lo));
}
__device__ __forceinline__ df sqr_u(df x) {
    const df c = two_prod(x.hi, x.hi);
    return mk(c.hi, __fmaf_rn(2.0f * x.hi, x.lo, c.lo));
}
// Products and quotients below 2^-102 in magnitude: the exact error terms
// of the pair arithmetic would be subnormal, so the pair loses precision.
// The lane is flagged for the native path instead.
#define AG_DF_MIN 1.9721522630525295e-31f   // 2^-102
__device__ __forceinline__ df ck(df v, bool& ok) {
    ok = ok && fabsf(v.hi) >= AG_DF_MIN;
    return v;
}
// Scale by an exact power of two.
__device__ __forceinline__ df scale(df x, float p2) { return mk(__fmul_rn(x.hi, p2), __fmul_rn(x.lo, p2)); }
// Sum where the first term dominates: |x.hi| >= |y.hi| (or x == 0), so the
// leading sum is exact by Fast2Sum (Dekker 1971) without the six-operation
// two-sum; the error is that of add_fast. Used where the caller's argument
// ranges prove the ordering.
__device__ __forceinline__ df add_quick(df x, df y) {
    const df s = fast_two_sum(x.hi, y.hi);
    const float v = __fadd_rn(__fadd_rn(x.lo, y.lo), s.lo);
    return fast_two_sum(s.hi, v);
}
__device__ __forceinline__ df add_quick(df x, float y) {
    const df s = fast_two_sum(x.hi, y);
    return fast_two_sum(s.hi, __fadd_rn(x.lo, s.lo));
}

// Hardware seeds (MUFU). The host branch exists only so the double-float
// algorithms can be checked by a host build of this header.
__device__ __forceinline__ float rcp_approx(float x) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}
__device__ __forceinline__ float rsqrt_approx(float x) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / sqrtf(x);
#endif
}

// Reciprocal: FP32 seed refined by two double-float Newton steps.
__device__ __forceinline__ df recip(df y) {
    float r = rcp_approx(y.hi);
    r = __fmaf_rn(r, __fmaf_rn(-y.hi, r, 1.0f), r);
    // e = 1 - y*r, computed exactly enough in double-float
    const df yr = mul(y, r);
    const float e = __fsub_rn(__fsub_rn(1.0f, yr.hi), yr.lo);
    return fast_two_sum(r, __fmul_rn(r, e));
}
// x / y: a float quotient q1 from a twice-refined reciprocal, then one
// correction from the residual x - y q1, formed exactly enough: y.hi q1 =
// p.hi + p.lo (two_prod), x.hi - p.hi is exact (Sterbenz: q1 is within 2^-23
// of the quotient) and the small terms join by fma.
__device__ __forceinline__ df div(df x, df y) {
    float r = rcp_approx(y.hi);
    r = __fmaf_rn(r, __fmaf_rn(-y.hi, r, 1.0f), r);
    r = __fmaf_rn(r, __fmaf_rn(-y.hi, r, 1.0f), r);   // twice: q1 within ~2^-24, so e's roundings stay at 2^-48 of q
    const float q1 = __fmul_rn(x.hi, r);
    const df p = two_prod(y.hi, q1);
    float e = __fsub_rn(x.hi, p.hi);
    e = __fsub_rn(e, p.lo);
    e = __fadd_rn(e, x.lo);
    e = __fmaf_rn(-y.lo, q1, e);
    return fast_two_sum(q1, __fmul_rn(e, r));
}

__device__ __forceinline__ bool gt(df a, df b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool lt(df a, df b) { return gt(b, a); }
__device__ __forceinline__ bool ge(df a, df b) { return !lt(a, b); }
__device__ __forceinline__ bool le(df a, df b) { return !gt(a, b); }
__device__ __forceinline__ bool eq(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool ne(df a, df b) { return !eq(a, b); }

// ---------------------------------------------------------------------------
// double <-> double-float, with integer operations only (no F2F).
// ---------------------------------------------------------------------------
// |x| in [2^-50, 2^60]: the input range of the double-float path. Squares and
// products of two inputs then stay within [2^-100, 2^120], where the exact
// error terms of the pair arithmetic are still normal floats (the generator
// checks every product it cannot prove to stay above 2^-102).
__device__ __forceinline__ bool in_range(double x) {
    const unsigned ah = (unsigned)__double2hiint(x) & 0x7fffffffu;
    return ah - (973u << 20) <= (111u << 20) - 1u;
}
// The split of a double, and its range test (the flag is cleared when |x|
// leaves [2^-50, 2^60]) from the same integer work: the float exponent of the
// head is the double's less 896, the tail's scale 2^(e-1075) is the head's
// exponent field less 52 (with the sign carried along).
__device__ __forceinline__ df from_double_ck(double x, bool& ok) {
    const unsigned h32 = (unsigned)__double2hiint(x);
    const unsigned l32 = (unsigned)__double2loint(x);
    const unsigned t = (h32 & 0x7fffffffu) - (896u << 20);
    ok = ok && t - (77u << 20) <= (111u << 20) - 1u;
    // hi: the top 24 significant bits (truncated), re-biased to float
    const unsigned hb = __funnelshift_l(l32, t, 3) | (h32 & 0x80000000u);
    // lo: the remaining 29 bits, rounded to a float and scaled by +-2^(ex-1075);
    // |lo| < ulp(hi), so the pair is used without renormalising
    const float lo = __fmul_rn(__uint2float_rn(l32 & 0x1fffffffu), __int_as_float((hb & 0xff800000u) - (52u << 23)));
    return mk(__int_as_float(hb), lo);
}
__device__ __forceinline__ df from_double(double x) {
    bool ok = true;
    return from_double_ck(x, ok);
}
// A normal float (or zero) as a double.
__device__ __forceinline__ double f2d(float f) {
    const unsigned b = (unsigned)__float_as_int(f);
    const unsigned e = (b >> 23) & 0xffu;
    const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    const double d = __hiloint2double((int)hi, (int)(b << 29));
    return e == 0u ? 0.0 : d;
}
// The reassembly uses the hardware float->double conversion: two FP64-pipe
// instructions instead of a dozen integer ones on the busier FP32/INT pipes
// (the FP64 pipe has room for a few operations per element at these rates).
__device__ __forceinline__ double to_double(df v) { return __dadd_rn((double)v.hi, (double)v.lo); }
// A result that reassembles exactly: finite, normal and away from underflow.
__device__ __forceinline__ bool out_ok(df v) {
    const unsigned e = ((unsigned)__float_as_int(v.hi) >> 23) & 0xffu;
    return e - 37u <= 216u;   // |hi| in [2^-90, 2^127)
}
// 0 < w < 2^54 as a double-float: the top 24 significant bits exactly, the
// rest rounded once (2^-48 relative).
__device__ __forceinline__ df from_u64(ag_u64 w) {
    const int sh = 40 - __clzll((long long)w);   // bits below the leading 24
    if (sh <= 0) return mk(__uint2float_rn((ag_u32)w), 0.0f);
    const float h = __fmul_rn(__uint2float_rn((ag_u32)(w >> sh)), __int_as_float((sh + 127) << 23));
    const float l = __uint2float_rn((ag_u32)(w & ((1ull << sh) - 1ull)));
    return fast_two_sum(h, l);
}
__device__ __forceinline__ float p2f(int k) { return __int_as_float((k + 127) << 23); }   // 2^k, |k| <= 126
// Round to nearest integer for |x| < 2^22 with one FP32 add (no conversion unit).
__device__ __forceinline__ float rint_f(float x) { return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f); }
__device__ __forceinline__ int rint_i(float x) { return __float_as_int(__fadd_rn(x, 12582912.0f)) - 0x4B400000; }

// ---------------------------------------------------------------------------
// Square root and reciprocal square root (Newton-Raphson, one double-float
// correction of a refined hardware seed).
// ---------------------------------------------------------------------------
// Hardware rsqrt seed refined once in FMA form to about 2^-24.5:
// y += (y/2) (1 - x y^2), the residual taken from an FMA.
__device__ __forceinline__ float rsqrt_seed(float x) {
    const float y = rsqrt_approx(x);
    const float e = __fmaf_rn(-__fmul_rn(x, y), y, 1.0f);
    return __fmaf_rn(__fmul_rn(0.5f, y), e, y);
}
// x > 0 (no zero, negative or NaN argument can reach it)
__device__ __forceinline__ df sqrt_pos_(df x) {
    const float y = rsqrt_seed(x.hi);
    const float s = __fmul_rn(x.hi, y);
    const df p = two_prod(s, s);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, p.hi), p.lo), x.lo);
    return fast_two_sum(s, __fmul_rn(r, 0.5f * y));
}
// Any argument: a negative or NaN one makes the seed NaN and with it the
// pair; zero (where seed times argument is 0 x inf) keeps its own branch.
__device__ __forceinline__ df sqrt_(df x) {
    const df res = sqrt_pos_(x);
    return x.hi == 0.0f ? mk(0.0f, 0.0f) : res;
}
__device__ __forceinline__ df sqrt_nn_(df x) { return sqrt_(x); }
// One Newton step on a float seed y: e = 1 - x y^2 and rsqrt x = y (1 + e/2).
// y^2 = p + q exactly (two_prod); x.hi p is within 2^-22 of 1, so fma(-x.hi,
// p, 1) carries e to 2^-24 of itself and the two smaller products join it by
// fma; the correction y e / 2 is ~2^-23 of y, so the result is good to ~2^-47.
__device__ __forceinline__ df rsqrt_(df x) {
    const float y = rsqrt_seed(x.hi);
    const df yy = two_prod(y, y);
    float e = __fmaf_rn(-x.hi, yy.hi, 1.0f);
    e = __fmaf_rn(-x.hi, yy.lo, e);
    e = __fmaf_rn(-x.lo, yy.hi, e);
    // x.hi <= 0, NaN or +inf make the seed or the residual NaN, so the pair is
    // NaN there without a test (and such lanes take the native path)
    return fast_two_sum(y, __fmul_rn(__fmul_rn(y, e), 0.5f));
}

// ---------------------------------------------------------------------------
// exp: x = (64k + j) ln2/64 + r, |r| <= ln2/128; e^x = 2^k 2^(j/64) e^r.
// ---------------------------------------------------------------------------
// The flag is cleared outside -70 < x < 87, where 2^k leaves the float range
// or the result's low part would be subnormal (the native lane computes it).
__device__ __forceinline__ df exp_(df x, bool& ok) {
    ok = ok && x.hi > -70.0f && x.hi < 87.0f;
    const float mf = rint_f(__fmul_rn(x.hi, AG_INV_LN2_64));
    const int m = rint_i(__fmul_rn(x.hi, AG_INV_LN2_64));
    const float r1 = __fmaf_rn(-mf, AG_LN2_64_1, x.hi);   // exact (Sterbenz)
    df r = two_sum(r1, x.lo);
    r = sub(r, two_prod(mf, AG_LN2_64_2));
    r = add(r, __fmul_rn(-mf, AG_LN2_64_3));
    // e^r - 1 = r + r^2/2 + r^3 (1/6 + r/24 + r^2/120)
    const float rh = r.hi;
    const float tail = __fmul_rn(__fmul_rn(rh, __fmul_rn(rh, rh)),
                                 __fmaf_rn(rh, __fmaf_rn(rh, 8.33333333e-3f, 4.16666667e-2f), 1.66666667e-1f));
    // |r| <= ln2/128, so each sum below is led by its first term
    df p = add_quick(r, scale(sqr(r), 0.5f));
    p = add_quick(p, tail);
    const int j = m & 63;
    int k = m >> 6;
    const df T = mk(__ldg(&kExp2TabHi[j]), __ldg(&kExp2TabLo[j]));
    const df res = add_quick(T, mul(T, p));
    k = k < -126 ? -126 : (k > 126 ? 126 : k);
    return scale(res, p2f(k));
}

// ---------------------------------------------------------------------------
// log: y = 2^e m, m in [0.75, 1.5), i = round(128 (m - 1)), c_i ~ 1/(1 + i/128)
// (c_0 = 1), t = y 2^-e c_i - 1 (|t| < 2^-7), log y = e ln2 - log c_i + log(1+t).
// log_s(s, x) is log(s + x) for s in {0, 1}: log for s = 0, log1p for s = 1,
// with t formed from s and x separately so 1 + x is never rounded.
// ---------------------------------------------------------------------------
// log(1+t) for |t| <= 2^-10.6: t - t^2/2 in double-float, the rest
// t^2 (t/3 - t^2/4 + t^3/5) in float (at most 2^-47.6 relative to t).
__device__ __forceinline__ df log1p_poly(df t) {
    // h = -t^2/2 as an unnormalised pair: -t.hi^2/2 rounded, its exact error
    // and -t.hi t.lo; r = t^2 q = (hh + hl) (-2 q), the -2 folded into q (r
    // needs t^2 to float accuracy, so the t.lo part of h joins it)
    const float th = t.hi;
    const float u = __fmul_rn(-0.5f, th);   // exact
    const float hh = __fmul_rn(th, u);
    const float hl = __fmaf_rn(-th, t.lo, __fmaf_rn(th, u, -hh));
    const float r = __fmul_rn(__fadd_rn(hh, hl),
                              __fmul_rn(th, __fmaf_rn(th, __fmaf_rn(th, -0.4f, 0.5f), -0.666666667f)));
    return add_quick(add_quick(t, mk(hh, hl)), r);
}
// log_s(s, x) for s + x > 0 with 2^-120 < s + x < 2^120 known in advance
// (checked = false) skips the validity test. MODE selects how the reduced
// argument t = s A - 1 + x A is formed: 0 for log (s = 0: x.hi A is within
// 2^-10 of 1, so x.hi A - 1 is exact by Sterbenz), 1 for log1p (s = 1:
// A - 1 as an exact two-sum), 2 for s in {0, 1} at run time where s A - 1 is
// a single exact FMA (s = 1 only with 1/2 <= s + x < 1, A in [2/3, 2]).
enum { LOG_S0 = 0, LOG_S1 = 1, LOG_SRT = 2 };
template <bool checked = true, int MODE = LOG_S1>
__device__ __forceinline__ df log_s(float s, df x) {
    const float yh = __fadd_rn(s, x.hi);
    const int bits = __float_as_int(yh);
    int e = ((bits >> 23) & 0xff) - 127;
    int mb = (bits & 0x007fffff) | 0x3f800000;
    if (bits & 0x00400000) {   // m >= 1.5: use m/2 and e+1
        mb -= 0x00800000;
        e += 1;
    }
    const float m = __int_as_float(mb);
    const int i = rint_i(__fmaf_rn(m, 1024.0f, -1024.0f)) + AG_LOG_TAB_OFF;   // (m - 1) 1024, exact
    const f4 cl = ld4(kLogCL, i);
    const float c = cl.x;
    const float A = __int_as_float((int)((unsigned)__float_as_int(c) - ((unsigned)e << 23)));   // c 2^-e, exact for valid e
    // x A = p + (x.lo A + p.lo), the pair left unnormalised for the sum
    const df p = two_prod(x.hi, A);
    const float pl = __fmaf_rn(x.lo, A, p.lo);
    df t;
    if (MODE == LOG_S0) {
        t = fast_two_sum(__fsub_rn(p.hi, 1.0f), pl);
    } else if (MODE == LOG_SRT) {
        const df u = two_sum(__fmaf_rn(s, A, -1.0f), p.hi);
        t = fast_two_sum(u.hi, __fadd_rn(pl, u.lo));
    } else {
        // B = A - 1 exactly; B.lo = 0 whenever B and x A can cancel (c_i - 1
        // is exact by Sterbenz for e = 0), so t keeps 2^-48 of itself there;
        // for e != 0 the result is >= 0.29 in magnitude and an error of 2^-48
        // of the terms is 2^-46.5 of it
        const df B = two_sum(A, -1.0f);
        const df u = two_sum(B.hi, p.hi);
        t = fast_two_sum(u.hi, __fadd_rn(__fadd_rn(B.lo, pl), u.lo));
    }
    const df L = mk(cl.y, cl.z);
    // e ln2 from a table covering every e the bits above can give (out-of-range
    // e is flagged below)
    const int ei = e + AG_LN2_TAB_OFF;
#ifdef __CUDA_ARCH__
    const float2 ep = __ldg(reinterpret_cast<const float2*>(kLn2Mul) + ei);
    const df E = mk(ep.x, ep.y);
#else
    const df E = mk(kLn2Mul[2 * ei], kLn2Mul[2 * ei + 1]);
#endif
    // |E| >= ln2 > |L + log1p(t)| except for e == 0 (E = 0), |L| >= 2^-10.6
    // >= |t| except for i == 0 (L = 0): each sum is led by its first term.
    df res;
    if (MODE == LOG_SRT) {
        // The Box-Muller logarithm (halved again by the square root that
        // follows): one chain E + L + t + h, h = -t^2/2 as an unnormalised
        // pair, with every low part and r = t^2 (t/3 - t^2/4 + t^3/5) gathered
        // into one float. About a quarter of the operations of the two
        // renormalised sums below, at a few per cent more mean error.
        const float th = t.hi;
        const float uu = __fmul_rn(-0.5f, th);
        const float hh = __fmul_rn(th, uu);
        const float hl = __fmaf_rn(-th, t.lo, __fmaf_rn(th, uu, -hh));
        const float r = __fmul_rn(__fadd_rn(hh, hl),
                                  __fmul_rn(th, __fmaf_rn(th, __fmaf_rn(th, -0.4f, 0.5f), -0.666666667f)));
        const df a1 = fast_two_sum(E.hi, L.hi);
        const df a2 = fast_two_sum(a1.hi, th);
        const df a3 = fast_two_sum(a2.hi, hh);   // |h| <= 2^-11.6 |t|
        const float lo = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(a1.lo, a2.lo), __fadd_rn(a3.lo, E.lo)),
                                             __fadd_rn(L.lo, t.lo)), __fadd_rn(hl, r));
        res = fast_two_sum(a3.hi, lo);
    } else {
        res = add_quick(E, add_quick(L, log1p_poly(t)));
    }
    if (!checked) return res;
    const bool valid = yh > 0.0f && e > -120 && e < 120;
    return valid ? res : mk(__int_as_float(0x7fc00000), 0.0f);
}
__device__ __forceinline__ df log_(df x) { return log_s<true, LOG_S0>(0.0f, x); }
__device__ __forceinline__ df log1p_(df x) { return log_s<true, LOG_S1>(1.0f, x); }
// log1p of an argument known to be >= 0 and below 2^60 (an input in the
// double-float range, or an expression of such inputs that cannot grow past it)
__device__ __forceinline__ df log1p_nn_(df x) { return log_s<false, LOG_S1>(1.0f, x); }

// ---------------------------------------------------------------------------
// sin/cos: r in [-pi/4, pi/4] (a little beyond is fine) split as r = j/2048 + t
// with |t| <= 2^-12; with S_j, C_j = sin, cos(j/2048) from a table,
// sin r = S_j (1 + cm1) + C_j st and cos r = C_j (1 + cm1) - S_j st, where
// st = sin t = t + t^3 (-1/6 + t^2/120) and cm1 = cos t - 1 = t^2 (-1/2 + t^2/24).
// For |t| <= 2^-12 the cubic and quadratic terms are below 2^-26.6 of t and of
// 1, so they are computed in float from t.hi; only t and the products with
// the table values are double-float.
// ---------------------------------------------------------------------------
// One output of sin/cos at x = q pi/2 + r: sin x is +-sin r or +-cos r by
// quadrant, and both are A (1 + cm1) + B st with the table pair (A, B) =
// (S_j, C_j) for sin r and (C_j, -S_j) for cos r, so only the wanted one is
// evaluated.
// The table step for x = q pi/2 + a + t, with sc = (sin a, cos a) from a table.
__device__ __forceinline__ df trig_tail(const f4& sc, df t, int q, bool want_cos) {
    const float th = t.hi;
    const float th2 = __fmul_rn(th, th);
    const float cubic = __fmul_rn(__fmul_rn(th, th2), __fmaf_rn(th2, 8.33333333e-3f, -1.66666667e-1f));
    const float cm1 = __fmul_rn(th2, __fmaf_rn(th2, 4.16666667e-2f, -0.5f));
    const int qq = (q + (want_cos ? 1 : 0)) & 3;   // cos x = sin(x + pi/2)
    const bool odd = qq & 1;
    const df A = odd ? mk(sc.z, sc.w) : mk(sc.x, sc.y);
    const df B = odd ? mk(-sc.x, -sc.y) : mk(sc.z, sc.w);
    // |A| >= sin(2^-11) >= 2 |B t| for j != 0, and A = 0 at j = 0 for sin r:
    // the sum is led by A
    const df v = add_quick(add_quick(A, mul_u(B, t)), __fmaf_rn(A.hi, cm1, __fmul_rn(B.hi, cubic)));
    return (qq & 2) ? neg(v) : v;
}
__device__ __forceinline__ df trig_core(df r, int q, bool want_cos) {
    int j = rint_i(__fmul_rn(r.hi, 2048.0f));
    j = j < -AG_SC_TAB_OFF ? -AG_SC_TAB_OFF : (j > AG_SC_TAB_OFF ? AG_SC_TAB_OFF : j);   // NaN-safe index
    const float jf = (float)j;
    const df t = fast_two_sum(__fsub_rn(r.hi, __fmul_rn(jf, 4.8828125e-4f)), r.lo);   // exact first difference
    return trig_tail(ld4(kSinCos2048, j + AG_SC_TAB_OFF), t, q, want_cos);
}
// Cody-Waite reduction by pi/2; valid for |k| < 4096, flagged otherwise.
__device__ __forceinline__ df dfc(double x);

#ifdef __CUDA_ARCH__
__device__ __forceinline__ ag_u64 umulhi64(ag_u64 a, ag_u64 b) { return __umul64hi(a, b); }
#else
inline ag_u64 umulhi64(ag_u64 a, ag_u64 b) { return (ag_u64)(((unsigned __int128)a * b) >> 64); }
#endif

// Payne-Hanek reduction (Payne & Hanek 1983) of a float h with 6000 <= |h| <
// 2^24, in 64-bit integer arithmetic: |h| = m 2^E with a 24-bit integer m and
// E in [-11, 0]; |h| 2/pi = m W 2^(E-192) with W = 2/pi to 192 bits, so the
// quadrant and 128 fraction bits come out of the three 64x64 products m W_i.
// Returns |h| - k pi/2 (a double-float, |.| <= pi/4) and k.
__device__ __forceinline__ df reduce_ph(float h, int& k, bool& ok) {
    const unsigned b = (unsigned)__float_as_int(h);
    const ag_u64 m = (ag_u64)((b & 0x7fffffu) | 0x800000u);
    int sh = 150 - (int)((b >> 23) & 0xffu);   // -E
    ok = ok && sh >= 0 && sh <= 11;
    sh = sh < 0 ? 0 : (sh > 11 ? 11 : sh);
    // m W from bit 64 up, as (a2:a1:a0)
    const ag_u64 p2h = umulhi64(m, AG_2OPI_W2);
    const ag_u64 p1l = m * AG_2OPI_W1, p1h = umulhi64(m, AG_2OPI_W1);
    const ag_u64 p0l = m * AG_2OPI_W0, p0h = umulhi64(m, AG_2OPI_W0);
    const ag_u64 a0 = p1l + p2h;
    const ag_u64 c0 = a0 < p1l ? 1ull : 0ull;
    ag_u64 a1 = p0l + p1h;
    ag_u64 c1 = a1 < p0l ? 1ull : 0ull;
    a1 += c0;
    c1 += a1 < c0 ? 1ull : 0ull;
    const ag_u64 a2 = p0h + c1;
    // the binary point sits sh bits into a2: integer part, then 128 fraction bits
    ag_u64 ip = a2 >> sh;
    ag_u64 fh = sh ? (a2 << (64 - sh)) | (a1 >> sh) : a1;
    ag_u64 fl = sh ? (a1 << (64 - sh)) | (a0 >> sh) : a0;
    // to the nearest quadrant: a fraction >= 1/2 becomes negative
    const bool up = (fh >> 63) != 0;
    ip += up ? 1ull : 0ull;
    if (up) {
        fl = ~fl + 1ull;
        fh = ~fh + (fl == 0 ? 1ull : 0ull);
    }
    // |fraction| = (fh:fl) 2^-128, normalised: top 48 bits as a double-float
    const int lz = fh ? __clzll((long long)fh) : 64 + __clzll((long long)(fl | 1ull));
    ok = ok && lz < 78;   // |r| >= 2^-78: otherwise too close to k pi/2 for the float exponent range
    const int l = lz < 78 ? lz : 77;
    const ag_u64 top = l < 64 ? (l ? (fh << l) | (fl >> (64 - l)) : fh) : (fl << (l - 64));
    const float th = __fmul_rn(__uint2float_rn((ag_u32)(top >> 40)), p2f(-24 - l));
    const float tl = __fmul_rn(__uint2float_rn((ag_u32)((top >> 16) & 0xffffffu)), p2f(-48 - l));
    df f = fast_two_sum(th, tl);
    f = mul(f, mk(AG_PIO2_HI, AG_PIO2_LO));
    k = (int)(ip & 3ull);
    return up ? neg(f) : f;
}

// |x| < 6000: Cody-Waite in float (three-part pi/2, exact products for |k| <
// 4096); 6000 <= |x| < 2^24: Payne-Hanek in integers; beyond, flagged (the
// native lane reduces it).
__device__ __forceinline__ df trig_(df x, bool want_cos, bool& ok) {
    const float ax = fabsf(x.hi);
    df r;
    int q;
    if (ax < 6000.0f) {
        const float kf = rint_f(__fmul_rn(x.hi, AG_TWO_OVER_PI));
        const float r1 = __fmaf_rn(-kf, AG_PIO2_1, x.hi);
        r = two_sum(r1, x.lo);
        r = sub(r, two_prod(kf, AG_PIO2_2));
        r = add(r, __fmul_rn(-kf, AG_PIO2_3));
        q = rint_i(__fmul_rn(x.hi, AG_TWO_OVER_PI));
    } else {
        int k;
        r = reduce_ph(ax, k, ok);
        if (x.hi < 0.0f) {
            r = neg(r);
            k = -k;
        }
        r = add(r, x.lo);   // x - k pi/2 = (hi - k pi/2) + lo
        q = k;
        // |lo| can reach ulp(hi)/2, up to 1/2 below 2^24: bring r back into [-pi/4, pi/4]
        if (r.hi > 0.78539816f) {
            r = sub(r, mk(AG_PIO2_HI, AG_PIO2_LO));
            q += 1;
        } else if (r.hi < -0.78539816f) {
            r = add(r, mk(AG_PIO2_HI, AG_PIO2_LO));
            q -= 1;
        }
    }
    return trig_core(r, q, want_cos);
}
__device__ __forceinline__ df sin_(df x, bool& ok) { return trig_(x, false, ok); }
__device__ __forceinline__ df cos_(df x, bool& ok) { return trig_(x, true, ok); }
// sin(pi v): exact reduction v = q/2 + r, |r| <= 1/4, then sin/cos of pi r.
__device__ __forceinline__ df sinpi_(df v) {
    const float qf = rint_f(__fmul_rn(v.hi, 2.0f));
    const df r = fast_two_sum(__fsub_rn(v.hi, __fmul_rn(qf, 0.5f)), v.lo);
    return trig_core(mul(r, mk(AG_PI_HI, AG_PI_LO)), rint_i(__fmul_rn(v.hi, 2.0f)), false);
}

// ---------------------------------------------------------------------------
// Philox draws as double-floats. Uniform: (2w+1) 2^-33 is exact in a
// double-float, so uniform(lo, hi) fills with power-of-two ranges are
// bit-exact. The normal draw (Box-Muller) is in ag_emu64_bm.cuh, which plans
// with normal leaves include.
// ---------------------------------------------------------------------------
__device__ __forceinline__ df draw01_df(ag_u64 seed, ag_u32 g, ag_u32 c) {
    const ag_u32 w = ag::philox_block(seed, g, c).x;
    return scale(from_u64(2ull * w + 1ull), p2f(-33));
}

// ---------------------------------------------------------------------------
// Scalars, simple nodes and the bridge to native FP64 for functions without a
// double-float kernel (each costs FP64-pipe work, like the native plan).
// ---------------------------------------------------------------------------
__device__ __forceinline__ df dfc(double x) {   // any double (runtime scalars, literals)
    const float h = __double2float_rn(x);
    const float l = isfinite(h) ? __double2float_rn(x - (double)h) : 0.0f;
    return mk(h, l);
}
// |x|: |hi|, and lo with the sign of hi taken off
__device__ __forceinline__ df abs_(df x) {
    return mk(fabsf(x.hi), __int_as_float(__float_as_int(x.lo) ^ (__float_as_int(x.hi) & (int)0x80000000)));
}
__device__ __forceinline__ df sign_(df x) {
    return mk(x.hi > 0.0f ? 1.0f : (x.hi < 0.0f ? -1.0f : 0.0f), 0.0f);
}
__device__ __forceinline__ df min_(df a, df b) { return lt(b, a) ? b : a; }
__device__ __forceinline__ df max_(df a, df b) { return gt(b, a) ? b : a; }
__device__ __forceinline__ double as_d(df x) { return (double)x.hi + (double)x.lo; }
#define AG_E64_NATIVE1(NAME)                                                                   \
    __device__ __forceinline__ df nat_##NAME(df x) { return dfc(ag::f_##NAME(as_d(x))); }
#define AG_E64_NATIVE2(NAME)                                                                   \
    __device__ __forceinline__ df nat_##NAME(df a, df b) { return dfc(ag::f_##NAME(as_d(a), as_d(b))); }
AG_E64_NATIVE1(expm1)
AG_E64_NATIVE1(exp2)
AG_E64_NATIVE1(log2)
AG_E64_NATIVE1(log10)
AG_E64_NATIVE1(tan)
AG_E64_NATIVE1(asin)
AG_E64_NATIVE1(acos)
AG_E64_NATIVE1(atan)
AG_E64_NATIVE1(tanh)
AG_E64_NATIVE1(sinh)
AG_E64_NATIVE1(cosh)
AG_E64_NATIVE1(floor)
AG_E64_NATIVE1(ceil)
AG_E64_NATIVE1(trunc)
AG_E64_NATIVE1(cbrt)
AG_E64_NATIVE1(erf)
AG_E64_NATIVE2(pow)
AG_E64_NATIVE2(atan2)
AG_E64_NATIVE2(hypot)
#undef AG_E64_NATIVE1
#undef AG_E64_NATIVE2

}  // namespace e64
}  // namespace ag
