// ag_tf64.cuh -- FP64-grade expression math on the FP32 and integer pipes.
//
// Included by generated kernels lowered with math = 3. The double-float
// lowering (ag_emu64.cuh, math = 1) carries about 48 significant bits, tens
// of double ulps short of the FP64 contract; the native pipe meets the
// contract at a few per cent of HBM bandwidth. Here every double is split
// exactly into three floats (24 + 23 + 6 significant bits, integer operations
// only), the expression is evaluated in triple-float arithmetic (about 72
// bits, of which the operations keep well over 60), and each output is
// reassembled into a double with two FP64 additions, one rounding of a value
// already exact to far below half an ulp.
//
// Representation: v = x + y + z with |y| of the order of ulp(x) and |z| of
// the order of 2^-24 |y|. The first two levels are combined by error-free
// transformations (two-sum, Fast2Sum, FMA two-product); the third is
// accumulated with plain float operations, whose roundings (2^-24 of a term
// of 2^-47 of the value) stay near 2^-71. The components are not kept
// strictly non-overlapping: every operation below accepts a y up to a few
// ulps of x and a z up to a few ulps of y.
//
// Range: inputs with magnitudes in [2^-40, 2^60] (and products the generator
// cannot prove to stay above 2^-80) keep every component a normal float;
// other lanes, non-finite or out-of-range outputs, and the functions without
// a triple-float kernel (tan, the inverse trigonometric and hyperbolic
// functions, pow and the rest) are computed with native FP64, so range and
// special values keep FP64 semantics.
//
// Methods (published; own code): Knuth two-sum, Dekker Fast2Sum, FMA
// two-product; Newton-Raphson square root, reciprocal square root and
// reciprocal, each a double-float result from ag_emu64.cuh refined by one
// step whose residual is formed exactly enough in triple-float; the
// table-driven logarithm of Tang (1990) with the reduction points of the
// double-float kernel and a third float on every table value; the
// table-driven exponential of Tang (1989); sine and cosine (ag_tf64_trig.cuh)
// by a four-part Cody-Waite reduction by pi/2 and a table of sin and cos at
// j/2048 (tables by gen_tf64_tables.py).
#pragma once

#include "ag_emu64.cuh"
#include "ag_tf64_tables.cuh"

namespace ag {
namespace t64 {

using e64::df;
using e64::fast_two_sum;
using e64::mk;
using e64::two_prod;
using e64::two_sum;

struct tf {
    float x, y, z;
};

__device__ __forceinline__ tf mk3(float x, float y, float z) {
    tf r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
__device__ __forceinline__ tf from_df(df v) { return mk3(v.hi, v.lo, 0.0f); }
__device__ __forceinline__ tf neg(tf a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ tf scale(tf a, float p2) {
    return mk3(__fmul_rn(a.x, p2), __fmul_rn(a.y, p2), __fmul_rn(a.z, p2));
}

// ---------------------------------------------------------------------------
// Arithmetic.
// ---------------------------------------------------------------------------
// a + b, any signs. The sum of the leading floats and of the second floats
// are exact pairs; their errors and the third floats form the third level.
// Under cancellation the result keeps an absolute error near 2^-71 of the
// larger operand.
__device__ __forceinline__ tf add(tf a, tf b) {
    const df s = two_sum(a.x, b.x);
    const df t = two_sum(a.y, b.y);
    const df u = two_sum(s.lo, t.hi);
    const float z = __fadd_rn(__fadd_rn(t.lo, u.lo), __fadd_rn(a.z, b.z));
    const df w = two_sum(s.hi, u.hi);
    return mk3(w.hi, w.lo, z);
}
__device__ __forceinline__ tf sub(tf a, tf b) { return add(a, neg(b)); }
// a + b for operands of one sign: |s.hi| is at least either leading float,
// so the last combination is a Fast2Sum.
__device__ __forceinline__ tf add_fast(tf a, tf b) {
    const df s = two_sum(a.x, b.x);
    const df t = two_sum(a.y, b.y);
    const df u = two_sum(s.lo, t.hi);
    const float z = __fadd_rn(__fadd_rn(t.lo, u.lo), __fadd_rn(a.z, b.z));
    const df w = fast_two_sum(s.hi, u.hi);
    return mk3(w.hi, w.lo, z);
}
// a + b where a leads: |a.x| >= |b.x| (or a.x = 0) and |a + b| >= |a| / 2, so
// the leading floats join by Fast2Sum and the result cannot cancel.
__device__ __forceinline__ tf add_lead(tf a, tf b) {
    const df s = fast_two_sum(a.x, b.x);
    const df t = two_sum(a.y, b.y);
    const df u = two_sum(s.lo, t.hi);
    const float z = __fadd_rn(__fadd_rn(t.lo, u.lo), __fadd_rn(a.z, b.z));
    const df w = fast_two_sum(s.hi, u.hi);
    return mk3(w.hi, w.lo, z);
}
// The reassembly into a double rounds x + y + z once whatever their overlap,
// so the root of a plan has no cheaper form here.
__device__ __forceinline__ tf add_fast_u(tf a, tf b) { return add_fast(a, b); }

// a b: the three products of the first two levels as exact pairs, the
// third-level products by FMA; the dropped terms are below 2^-70 of the
// product.
__device__ __forceinline__ tf mul(tf a, tf b) {
    const df p = two_prod(a.x, b.x);
    const df q1 = two_prod(a.x, b.y);
    const df q2 = two_prod(a.y, b.x);
    const float r = __fmaf_rn(a.y, b.y, __fmaf_rn(a.x, b.z, __fmul_rn(a.z, b.x)));
    const df s = two_sum(q1.hi, q2.hi);
    const df u = two_sum(p.lo, s.hi);
    const float z = __fadd_rn(__fadd_rn(__fadd_rn(q1.lo, q2.lo), __fadd_rn(s.lo, u.lo)), r);
    const df w = fast_two_sum(p.hi, u.hi);   // |u.hi| is about 2^-23 |p.hi| at most
    return mk3(w.hi, w.lo, z);
}
__device__ __forceinline__ tf mul(tf a, float f) {
    const df p = two_prod(a.x, f);
    const df q = two_prod(a.y, f);
    const df u = two_sum(p.lo, q.hi);
    const float z = __fmaf_rn(a.z, f, __fadd_rn(q.lo, u.lo));
    const df w = fast_two_sum(p.hi, u.hi);
    return mk3(w.hi, w.lo, z);
}
__device__ __forceinline__ tf sqr(tf a) {
    const df p = two_prod(a.x, a.x);
    const float x2 = __fmul_rn(2.0f, a.x);   // exact
    const df q = two_prod(x2, a.y);
    const float r = __fmaf_rn(a.y, a.y, __fmul_rn(x2, a.z));
    const df u = two_sum(p.lo, q.hi);
    const float z = __fadd_rn(__fadd_rn(q.lo, u.lo), r);
    const df w = fast_two_sum(p.hi, u.hi);
    return mk3(w.hi, w.lo, z);
}
// The square of a double-float as a triple-float (no third input float).
__device__ __forceinline__ tf sqr_df(df a) {
    const df p = two_prod(a.hi, a.hi);
    const df q = two_prod(__fmul_rn(2.0f, a.hi), a.lo);
    const df u = two_sum(p.lo, q.hi);
    const float z = __fmaf_rn(a.lo, a.lo, __fadd_rn(q.lo, u.lo));
    const df w = fast_two_sum(p.hi, u.hi);
    return mk3(w.hi, w.lo, z);
}
// Products read only by sums: the reassembly and every sum above take any
// overlap, so the same value serves.
__device__ __forceinline__ tf sqr_u(tf a) { return sqr(a); }

// Products below 2^-80 in magnitude would push the third float toward the
// subnormal range; such lanes take the native path.
#define AG_TF_MIN 8.2718061255302767e-25f   // 2^-80
__device__ __forceinline__ tf ck(tf v, bool& ok) {
    ok = ok && fabsf(v.x) >= AG_TF_MIN;
    return v;
}

// (x, y, z) with the overlap of y and z folded into y: y + z as an exact
// pair, then x with its leading part (two-sums, so x may be the smaller).
__device__ __forceinline__ tf renorm(tf v) {
    const df s = two_sum(v.y, v.z);
    const df w = two_sum(v.x, s.hi);
    return mk3(w.hi, w.lo, s.lo);
}

// Reciprocal: the double-float reciprocal (about 2^-47) refined by one Newton
// step r' = r + r e, e = 1 - y r. y r is within 2^-46 of 1, so 1 - x of the
// product is exact (Sterbenz) and its second and third floats join by
// subtractions that are exact or round at 2^-70.
__device__ __forceinline__ tf recip(tf y) {
    const df r = e64::recip(mk(y.x, y.y));
    const tf m = mul(y, from_df(r));
    const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, m.x), m.y), m.z);
    return mk3(r.hi, r.lo, __fmul_rn(r.hi, e));
}
__device__ __forceinline__ tf div(tf a, tf b) { return mul(a, recip(b)); }

// Comparisons by the sign of the difference: the leading float of a sum
// carries its sign unless the whole sum is zero at the first two levels.
__device__ __forceinline__ int sgn_(tf d) {
    const float v = d.x != 0.0f ? d.x : (d.y != 0.0f ? d.y : d.z);
    return v > 0.0f ? 1 : (v < 0.0f ? -1 : 0);
}
__device__ __forceinline__ bool gt(tf a, tf b) { return sgn_(sub(a, b)) > 0; }
__device__ __forceinline__ bool lt(tf a, tf b) { return sgn_(sub(a, b)) < 0; }
__device__ __forceinline__ bool ge(tf a, tf b) { return sgn_(sub(a, b)) >= 0; }
__device__ __forceinline__ bool le(tf a, tf b) { return sgn_(sub(a, b)) <= 0; }
__device__ __forceinline__ bool eq(tf a, tf b) { return sgn_(sub(a, b)) == 0; }
__device__ __forceinline__ bool ne(tf a, tf b) { return sgn_(sub(a, b)) != 0; }

// ---------------------------------------------------------------------------
// double <-> triple-float.
// ---------------------------------------------------------------------------
// The exact split of a double with |x| in [2^-40, 2^60] (the flag is cleared
// outside): x takes the implicit bit and the top 23 stored bits (the same
// integer work as the double-float split), y the next 23 bits and z the last
// 6, each made a float by the 2^23 exponent trick (no conversion unit) and
// scaled by a power of two built from x's exponent field.
__device__ __forceinline__ tf from_double_ck(double v, bool& ok) {
    const unsigned h32 = (unsigned)__double2hiint(v);
    const unsigned l32 = (unsigned)__double2loint(v);
    const unsigned t = (h32 & 0x7fffffffu) - (896u << 20);
    ok = ok && t - (87u << 20) <= (101u << 20) - 1u;   // double exponent in [-40, 60]
    const unsigned hb = __funnelshift_l(l32, t, 3) | (h32 & 0x80000000u);
    const unsigned se = hb & 0xff800000u;   // sign and exponent field of x
    const float my = __fsub_rn(__int_as_float((int)(0x4B000000u | ((l32 >> 6) & 0x7fffffu))), 8388608.0f);
    const float mz = __fsub_rn(__int_as_float((int)(0x4B000000u | (l32 & 63u))), 8388608.0f);
    // bit k of the stored mantissa weighs 2^(e - 52 + k): y's lowest bit is
    // bit 6, z's bit 0
    const float y = __fmul_rn(my, __int_as_float((int)(se - (46u << 23))));
    const float z = __fmul_rn(mz, __int_as_float((int)(se - (52u << 23))));
    return mk3(__int_as_float((int)hb), y, z);
}
// Any double (runtime scalars, literals, native results): the split by
// conversions on the FP64 pipe, exact for normal values.
__device__ __forceinline__ tf dfc(double v) {
    const float x = __double2float_rn(v);
    if (!isfinite(x)) return mk3(x, 0.0f, 0.0f);
    const double r = v - (double)x;
    const float y = __double2float_rn(r);
    return mk3(x, y, __double2float_rn(r - (double)y));
}
// y + z in a double is exact whenever their exponents lie within 29 of each
// other, and otherwise off by at most 2^-53 of y (about 2^-77 of x): the
// result is x + y + z rounded once, to far below half an ulp.
__device__ __forceinline__ double to_double(tf v) {
    return __dadd_rn((double)v.x, __dadd_rn((double)v.y, (double)v.z));
}
__device__ __forceinline__ double as_d(tf v) { return to_double(v); }
// An output whose three floats were all normal: |x| in [2^-80, 2^127).
__device__ __forceinline__ bool out_ok(tf v) {
    const unsigned e = ((unsigned)__float_as_int(v.x) >> 23) & 0xffu;
    return e - 47u <= 206u;
}

// ---------------------------------------------------------------------------
// Square root and reciprocal square root.
// ---------------------------------------------------------------------------
// a > 0. s = the double-float root (about 2^-47), then s' = s + (a - s^2)
// y/2 with y ~ 1/sqrt(a) the float seed. The residual is about 2^-47 a and is
// needed to 2^-12 of itself: a.x - s.hi^2 is exact (Sterbenz), and the terms
// of the second level, each up to 2^-23 a and cancelling to the residual, are
// summed by two-sums.
__device__ __forceinline__ tf sqrt_pos_(tf a) {
    const float y = e64::rsqrt_seed(a.x);
    const float s0 = __fmul_rn(a.x, y);
    const df p0 = two_prod(s0, s0);
    const float r0 = __fadd_rn(__fsub_rn(__fsub_rn(a.x, p0.hi), p0.lo), a.y);
    const float hy = __fmul_rn(0.5f, y);
    const df s = fast_two_sum(s0, __fmul_rn(r0, hy));
    const df P = two_prod(s.hi, s.hi);
    const df Q = two_prod(__fmul_rn(2.0f, s.hi), s.lo);
    const df e1 = two_sum(__fsub_rn(a.x, P.hi), a.y);
    const df e2 = two_sum(e1.hi, -P.lo);
    const df e3 = two_sum(e2.hi, -Q.hi);
    const float small = __fsub_rn(__fadd_rn(__fadd_rn(e1.lo, e2.lo), __fadd_rn(e3.lo, a.z)),
                                  __fmaf_rn(s.lo, s.lo, Q.lo));
    const float R = __fadd_rn(e3.hi, small);
    return mk3(s.hi, s.lo, __fmul_rn(R, hy));
}
__device__ __forceinline__ tf sqrt_(tf a) {
    const tf r = sqrt_pos_(a);
    return a.x == 0.0f ? mk3(0.0f, 0.0f, 0.0f) : r;
}
__device__ __forceinline__ tf sqrt_nn_(tf a) { return sqrt_(a); }
// a > 0. y = the double-float rsqrt (about 2^-47), then y' = y + y e / 2 with
// e = 1 - a y^2 formed like the reciprocal's residual.
__device__ __forceinline__ tf rsqrt_(tf a) {
    const df y = e64::rsqrt_(mk(a.x, a.y));
    const tf m = mul(a, sqr_df(y));
    const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, m.x), m.y), m.z);
    return mk3(y.hi, y.lo, __fmul_rn(__fmul_rn(y.hi, e), 0.5f));
}

// ---------------------------------------------------------------------------
// log and log1p: y = s + a = 2^e m, m in [0.75, 1.5), i = round(1024 (m - 1)),
// A = c_i 2^-e, t = s A - 1 + a A (|t| <= 2^-10.6), and
// log y = e ln2 - log c_i + log1p(t), log1p(t) = t + t^2 Q(t) with
// Q = -1/2 + t/3 - t^2/4 + t^3/5 - t^4/6 + t^5/7 (the next term is below
// 2^-66 of t). t^2 Q is about 2^-12 of t, so it is formed in double-float
// (2^-46 of itself, 2^-58 of t) with the coefficient 1/3 as a float pair.
// ---------------------------------------------------------------------------
enum { LOG_S0 = 0, LOG_S1 = 1 };
template <bool checked, int MODE>
__device__ __forceinline__ tf log_s(float s, tf a) {
    const float yh = __fadd_rn(s, a.x);
    const int bits = __float_as_int(yh);
    int e = ((bits >> 23) & 0xff) - 127;
    int mb = (bits & 0x007fffff) | 0x3f800000;
    if (bits & 0x00400000) {   // m >= 1.5: use m/2 and e+1
        mb -= 0x00800000;
        e += 1;
    }
    const float m = __int_as_float(mb);
    const int i = e64::rint_i(__fmaf_rn(m, 1024.0f, -1024.0f)) + AG_TF_LOG_TAB_OFF;
    const e64::f4 cl = e64::ld4(kLogCL3, i);
    const float A = __int_as_float((int)((unsigned)__float_as_int(cl.x) - ((unsigned)e << 23)));   // c 2^-e, exact
    const tf aA = mul(a, A);
    tf t;
    if (MODE == LOG_S0) {
        // a A is within 2^-10 of 1: its leading float less 1 is exact
        const df d = two_sum(__fsub_rn(aA.x, 1.0f), aA.y);
        t = mk3(d.hi, d.lo, aA.z);
    } else {
        const df B = two_sum(A, -1.0f);   // A - 1 exactly
        t = add(mk3(B.hi, B.lo, 0.0f), aA);
    }
    // t's third float can be far above an ulp of its second when t is small
    // (a A within 2^-24 of 1 leaves a's third float beside a tiny leading
    // part), and the series below reads t's first two floats only
    t = renorm(t);
    // P = t^2 Q in double-float
    const float th = t.x;
    const df tt = mk(t.x, t.y);
    const float R = __fmaf_rn(th, __fmaf_rn(th, __fmaf_rn(th, 0.142857143f, -0.166666667f), 0.2f), -0.25f);
    const df G = e64::add_quick(mk(AG_TF_THIRD_HI, AG_TF_THIRD_LO), e64::mul(tt, R));
    const df Q = e64::add_quick(mk(-0.5f, 0.0f), e64::mul(tt, G));
    const df P = e64::mul(e64::sqr(tt), Q);
    // T = t + P: |P| < |t| / 2^11
    const df h = fast_two_sum(t.x, P.hi);
    const df k = two_sum(h.lo, t.y);
    const tf T = mk3(h.hi, k.hi, __fadd_rn(__fadd_rn(k.lo, t.z), P.lo));
    // e ln2 - log c_i, each from its table as three floats. |e ln2| >= ln2 >
    // 0.29 >= |log c_i| unless e = 0, and |-log c_i| >= 2^-10 >= 2 |T| unless
    // i = 0 (then the leading term is 0): both sums are led by their first term.
    const e64::f4 ep = e64::ld4(kLn2Mul3, e + AG_TF_LN2_TAB_OFF);
    const tf res = add_lead(add_lead(mk3(ep.x, ep.y, ep.z), mk3(cl.y, cl.z, cl.w)), T);
    if (!checked) return res;
    const bool valid = yh > 0.0f && e > -120 && e < 120;
    return valid ? res : mk3(__int_as_float(0x7fc00000), 0.0f, 0.0f);
}
__device__ __forceinline__ tf log_(tf a) { return log_s<true, LOG_S0>(0.0f, a); }
__device__ __forceinline__ tf log1p_(tf a) { return log_s<true, LOG_S1>(1.0f, a); }
// log1p of an argument known to be >= 0 and within the input range
__device__ __forceinline__ tf log1p_nn_(tf a) { return log_s<false, LOG_S1>(1.0f, a); }

// ---------------------------------------------------------------------------
// Simple nodes, Philox draws and the bridge to native FP64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ tf abs_(tf a) { return sgn_(a) < 0 ? neg(a) : a; }
__device__ __forceinline__ tf sign_(tf a) { return mk3((float)sgn_(a), 0.0f, 0.0f); }
__device__ __forceinline__ tf min_(tf a, tf b) { return lt(b, a) ? b : a; }
__device__ __forceinline__ tf max_(tf a, tf b) { return gt(b, a) ? b : a; }
// (2w + 1) 2^-33: exact in the first two floats.
__device__ __forceinline__ tf draw01_df(ag_u64 seed, ag_u32 g, ag_u32 c) {
    return from_df(e64::draw01_df(seed, g, c));
}
// Normals from the native FP64 Box-Muller draw (the reference's formula).
template <bool U = false>
__device__ __forceinline__ tf normal_df(ag_u64 seed, ag_u32 g, ag_u32 c) {
    return dfc(ag::normal_f64(seed, g, c));
}
// ---------------------------------------------------------------------------
// exp: x = k ln2/64 + r, |r| <= ln2/128, e^x = 2^(k >> 6) T_(k & 63) (1 + p),
// T_j = 2^(j/64) from a table of three floats, p = e^r - 1 = r + r^2 Q(r),
// Q = 1/2 + r/6 + r^2/24 + r^3/120 + r^4/720 + r^5/5040 (the next term is
// below 2^-66). r = x - k (ln2/64) with ln2/64 as three floats (k < 2^13, so
// the product is good to 2^-63 absolute, the sum exact to 2^-64). r^2 Q is at
// most 2^-16: formed in double-float (2^-46 of itself), with 1/6 and 1/24 as
// float pairs where their products with r sit within 2^-12 of the terms
// before them. The flag is cleared outside -55 < x < 87, where 2^(k >> 6) or
// the result's third float would leave the normal floats (the native lane
// computes those).
// ---------------------------------------------------------------------------
__device__ __forceinline__ tf exp_(tf x, bool& ok) {
    ok = ok && x.x > -55.0f && x.x < 87.0f;
    const float kx = __fmul_rn(x.x, AG_TF_INV_LN2_64);
    const float kf = e64::rint_f(kx);
    const int k = e64::rint_i(kx);
    const tf r = renorm(sub(x, mul(mk3(AG_TF_LN2_64_X, AG_TF_LN2_64_Y, AG_TF_LN2_64_Z), kf)));
    const df rr = mk(r.x, r.y);
    const float rh = r.x;
    const float J = __fmaf_rn(rh, __fmaf_rn(rh, 1.98412698e-4f, 1.38888889e-3f), 8.33333333e-3f);
    const df H = e64::add_quick(mk(AG_TF_24TH_HI, AG_TF_24TH_LO), __fmul_rn(rh, J));
    const df G = e64::add_quick(mk(AG_TF_SIXTH_HI, AG_TF_SIXTH_LO), e64::mul(rr, H));
    const df Q = e64::add_quick(mk(0.5f, 0.0f), e64::mul(rr, G));
    const df P = e64::mul(e64::sqr(rr), Q);
    // p = r + P: |P| <= r^2 < |r|
    const df h = fast_two_sum(r.x, P.hi);
    const df m = two_sum(h.lo, r.y);
    const tf p = mk3(h.hi, m.hi, __fadd_rn(__fadd_rn(m.lo, r.z), P.lo));
    const e64::f4 tv = e64::ld4(kExp2Tab3, k & 63);
    const tf T = mk3(tv.x, tv.y, tv.z);
    // T >= 1 leads T p (|p| < 2^-7)
    const tf res = add_lead(T, mul(T, p));
    int e = k >> 6;
    e = e < -126 ? -126 : (e > 126 ? 126 : e);
    return scale(res, e64::p2f(e));
}
#define AG_T64_NATIVE1(NAME)                                                                   \
    __device__ __forceinline__ tf nat_##NAME(tf x) { return dfc(ag::f_##NAME(as_d(x))); }
#define AG_T64_NATIVE2(NAME)                                                                   \
    __device__ __forceinline__ tf nat_##NAME(tf a, tf b) { return dfc(ag::f_##NAME(as_d(a), as_d(b))); }
AG_T64_NATIVE1(expm1)
AG_T64_NATIVE1(exp2)
AG_T64_NATIVE1(log2)
AG_T64_NATIVE1(log10)
AG_T64_NATIVE1(tan)
AG_T64_NATIVE1(asin)
AG_T64_NATIVE1(acos)
AG_T64_NATIVE1(atan)
AG_T64_NATIVE1(tanh)
AG_T64_NATIVE1(sinh)
AG_T64_NATIVE1(cosh)
AG_T64_NATIVE1(floor)
AG_T64_NATIVE1(ceil)
AG_T64_NATIVE1(trunc)
AG_T64_NATIVE1(cbrt)
AG_T64_NATIVE1(erf)
AG_T64_NATIVE2(pow)
AG_T64_NATIVE2(atan2)
AG_T64_NATIVE2(hypot)
#undef AG_T64_NATIVE1
#undef AG_T64_NATIVE2

}  // namespace t64
}  // namespace ag
