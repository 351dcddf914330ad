// ag_tf64_trig.cuh -- FP64-grade sine and cosine in triple-float arithmetic.
//
// Included by generated FP64-grade kernels (math = 3) with trigonometric
// nodes. x = q pi/2 + r with pi/2 in four parts (the first with 14 significant
// bits, so q P0 is exact for |q| < 2^10; about 87 bits in all); r = j/2048 + t
// with |t| <= 2^-12 and S_j, C_j = sin, cos(j/2048) from a table of three
// floats each; then, by quadrant, sin r = S (1 + cm1) + C st and
// cos r = C (1 + cm1) - S st with st = sin t = t (1 + c), c = -t^2/6 + t^4/120,
// and cm1 = cos t - 1 = -t^2/2 + t^4/24 (both corrections at most 2^-25, so
// double-float carries them to 2^-72).
//
// The reduction keeps every term exact: x.x - q P0 (Sterbenz), q P1 and q P2
// as two-products, and the terms of each level summed by two-sums, so r is
// good to about 2^-77 absolute. Lanes with |x| >= 2^10, or with |r| < 2^-22
// for q != 0 (x within 2^-22 of a nonzero multiple of pi/2, where 2^-77 would
// exceed 2^-55 of r), clear the range flag and are computed natively.
#pragma once

#include "ag_tf64.cuh"
#include "ag_tf64_trig_tables.cuh"

namespace ag {
namespace t64 {

// r = x - q pi/2, |r| <= pi/4 (a little beyond is fine).
__device__ __forceinline__ tf reduce_pio2(tf x, int& q, bool& ok) {
    const float qx = __fmul_rn(x.x, AG_TF_2OPI);
    const float qf = e64::rint_f(qx);
    q = e64::rint_i(qx);
    ok = ok && fabsf(x.x) < 1024.0f;
    const float a0 = __fmaf_rn(-qf, AG_TF_PIO2_0, x.x);   // exact: q P0 has <= 24 bits, Sterbenz
    const df p1 = two_prod(qf, AG_TF_PIO2_1);
    const df p2 = two_prod(qf, AG_TF_PIO2_2);
    const float p3 = __fmul_rn(qf, AG_TF_PIO2_3);
    // first level: a0 - q P1
    const df s = two_sum(a0, -p1.hi);
    // second level: s.lo, x.y, -p1.lo, -p2.hi, each summed exactly
    const df u = two_sum(x.y, -p1.lo);
    const df v = two_sum(s.lo, -p2.hi);
    const df w = two_sum(u.hi, v.hi);
    // third level: the errors of the second and the smallest terms, again by
    // two-sums; only the last roundings (2^-24 of 2^-62) are plain
    const df a = two_sum(u.lo, v.lo);
    const df b = two_sum(w.lo, x.z);
    const df c = two_sum(a.hi, b.hi);
    const float tail = __fadd_rn(__fadd_rn(__fadd_rn(a.lo, b.lo), c.lo), -__fadd_rn(p2.lo, p3));
    const df z = two_sum(c.hi, tail);
    // r = s.hi + w.hi + z.hi + z.lo, normalised (the parts can cancel)
    const df m = two_sum(w.hi, z.hi);
    const df n = two_sum(s.hi, m.hi);
    const df k = two_sum(n.lo, m.lo);
    const tf r = mk3(n.hi, k.hi, __fadd_rn(k.lo, z.lo));
    ok = ok && (q == 0 || fabsf(r.x) >= 2.384185791e-7f);   // 2^-22
    return renorm(r);
}

// One output of sin/cos at x = q pi/2 + r: by quadrant it is +-sin r or
// +-cos r, and both are A (1 + cm1) + B st with (A, B) = (S, C) for sin r and
// (C, -S) for cos r, so only the wanted one is evaluated.
__device__ __forceinline__ tf trig_(tf x, bool want_cos, bool& ok) {
    int q;
    const tf r = reduce_pio2(x, q, ok);
    const float jf = e64::rint_f(__fmul_rn(r.x, 2048.0f));
    int j = e64::rint_i(__fmul_rn(r.x, 2048.0f));
    j = j < -1664 ? -1664 : (j > 1664 ? 1664 : j);
    // t = r - j/2048: the leading difference is exact (Sterbenz, or j = 0)
    const tf t = renorm(mk3(__fmaf_rn(-jf, 4.8828125e-4f, r.x), r.y, r.z));
    const e64::f4 s0 = e64::ld4(kSinCos3, 2 * (j + AG_TF_SC_TAB_OFF));
    const e64::f4 s1 = e64::ld4(kSinCos3, 2 * (j + AG_TF_SC_TAB_OFF) + 1);
    const tf S = mk3(s0.x, s0.y, s0.z), C = mk3(s0.w, s1.x, s1.y);
    // st = t (1 + c), cm1 = -t^2/2 + t^4/24, both corrections in double-float
    const df tt = mk(t.x, t.y);
    const df t2 = e64::sqr(tt);
    const float t4 = __fmul_rn(t2.hi, t2.hi);
    const df c = e64::add_quick(e64::mul(t2, mk(-AG_TF_SIXTH_HI, -AG_TF_SIXTH_LO)), __fmul_rn(t4, 8.33333333e-3f));
    const df cm1 = e64::add_quick(e64::scale(t2, -0.5f), __fmul_rn(t4, 4.16666667e-2f));
    const df tc = e64::mul(tt, c);
    // st = t + t c: |t c| <= 2^-26 |t|
    const df h = fast_two_sum(t.x, tc.hi);
    const df g = two_sum(h.lo, t.y);
    const tf st = mk3(h.hi, g.hi, __fadd_rn(__fadd_rn(g.lo, t.z), tc.lo));
    const int quad = (q + (want_cos ? 1 : 0)) & 3;   // 0: sin r, 1: cos r, 2: -sin r, 3: -cos r
    const bool use_cos = quad & 1;
    const tf A = use_cos ? C : S;
    const tf B = use_cos ? neg(S) : C;
    // A leads: |A| >= sin(1/2048) > |B st| unless A = 0 (j = 0 for sin r);
    // A cm1 is 2^-25 of A at most
    const df Acm = e64::mul(mk(A.x, A.y), cm1);
    const tf v = add_lead(add_lead(A, mul(B, st)), mk3(Acm.hi, Acm.lo, 0.0f));
    return quad & 2 ? neg(v) : v;
}
__device__ __forceinline__ tf sin_(tf x, bool& ok) { return trig_(x, false, ok); }
__device__ __forceinline__ tf cos_(tf x, bool& ok) { return trig_(x, true, ok); }

}  // namespace t64
}  // namespace ag
