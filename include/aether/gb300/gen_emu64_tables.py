"""Generate ag_emu64_tables.cuh and ag_emu64_bm_tables.cuh: the tables and
split constants of the double-float (float hi + float lo) function kernels in
ag_emu64.cuh and of the Box-Muller draw in ag_emu64_bm.cuh.

Every value is computed here with mpmath at 200 bits and rounded twice to
float (hi = fl(v), lo = fl(v - hi)), so hi + lo carries about 48 bits.
Methods: table-driven exponential (Tang 1989), table-driven logarithm with an
exact reduction t = m*c - 1 (Tang 1990), sine/cosine by Cody-Waite reduction
by pi/2 plus a 1/32-spaced table (Cody & Waite 1980).

usage: python aether_gb300/csrc/device/gen_emu64_tables.py
"""

import os

import mpmath as mp
import numpy as np

mp.mp.prec = 200
HERE = os.path.dirname(os.path.abspath(__file__))


def f32(v):
    return float(np.float32(float(v)))


def split2(v):
    hi = f32(v)
    lo = f32(mp.mpf(v) - hi)
    return hi, lo


def split3(v):
    hi = f32(v)
    mid = f32(mp.mpf(v) - hi)
    lo = f32(mp.mpf(v) - hi - mid)
    return hi, mid, lo


def trunc_bits(v, bits):
    """v rounded toward zero to `bits` significant bits (a float)."""
    v = mp.mpf(v)
    e = mp.floor(mp.log(abs(v), 2))
    scale = mp.mpf(2) ** (bits - 1 - e)
    return f32(mp.floor(abs(v) * scale) / scale * mp.sign(v))


def fl(x):
    s = np.float32(x)
    r = repr(float(s))
    if "inf" in r or "nan" in r:
        raise ValueError(r)
    return "%sf" % np.format_float_scientific(s, precision=9, unique=False)


def main():
    out = ["// generated by gen_emu64_tables.py -- do not edit", "#pragma once", "namespace ag {", "namespace e64 {"]

    # --- exp: 2^(j/64) ----------------------------------------------------
    exp_hi, exp_lo = zip(*[split2(mp.power(2, mp.mpf(j) / 64)) for j in range(64)])
    out.append("__device__ const float kExp2TabHi[64] = {%s};" % ", ".join(fl(v) for v in exp_hi))
    out.append("__device__ const float kExp2TabLo[64] = {%s};" % ", ".join(fl(v) for v in exp_lo))
    ln2_64 = mp.log(2) / 64
    # Cody-Waite parts of ln2/64: the first with 11 significant bits so m*C1 is exact for |m| < 2^13.
    c1 = trunc_bits(ln2_64, 11)
    c2 = trunc_bits(ln2_64 - c1, 24)
    c3 = f32(ln2_64 - c1 - c2)
    out.append("#define AG_LN2_64_1 %s" % fl(c1))
    out.append("#define AG_LN2_64_2 %s" % fl(c2))
    out.append("#define AG_LN2_64_3 %s" % fl(c3))
    out.append("#define AG_INV_LN2_64 %s" % fl(64 / mp.log(2)))

    # --- log: m in [0.75, 1.5), i = round((m-1)*1024) in [-256, 512] --------
    # c_i ~ 1/m_i as a full float; c_0 = 1 exactly (no cancellation near 1).
    # |t| = |m c_i - 1| <= 2^-10.6, so log(1+t) needs only t - t^2/2 exactly.
    cs, lh, ll = [], [], []
    for i in range(-256, 513):
        if i == 0:
            c = 1.0
        else:
            c = f32(1 / (1 + mp.mpf(i) / 1024))
        cs.append(c)
        h, l = split2(-mp.log(mp.mpf(c)))
        lh.append(h)
        ll.append(l)
    out.append("#define AG_LOG_TAB_OFF 256")
    # packed (c_i, -log c_i hi, lo, 0): one 16-byte load per lookup
    packed = []
    for c, h, l in zip(cs, lh, ll):
        packed += [c, h, l, 0.0]
    out.append("__device__ __align__(16) const float kLogCL[%d] = {%s};" % (len(packed), ", ".join(fl(v) for v in packed)))
    ln2 = mp.log(2)
    # e ln2 for e in [-127, 128] as a float pair (the exponent part of a log)
    # e in [-129, 130]: every exponent the reduction can produce from a float's
    # bits (including NaN and infinity, +1 for the m >= 1.5 step), so the
    # index needs no clamp
    e_hi, e_lo = zip(*[split2(e * ln2) for e in range(-129, 131)])
    out.append("#define AG_LN2_TAB_OFF 129")
    e_pairs = [v for pair in zip(e_hi, e_lo) for v in pair]
    out.append("__device__ __align__(8) const float kLn2Mul[%d] = {%s};" % (len(e_pairs), ", ".join(fl(v) for v in e_pairs)))

    # --- sin/cos at j/2048, j in [-1664, 1664], packed (S hi, S lo, C hi, C lo) --
    # so one 16-byte load serves a lookup; |r - j/2048| <= 2^-12 leaves the
    # cubic and quadratic terms of the remainder exact enough in float.
    packed = []
    for j in range(-1664, 1665):
        a = mp.mpf(j) / 2048
        packed += list(split2(mp.sin(a))) + list(split2(mp.cos(a)))
    # 2/pi as a 192-bit fraction, three 64-bit words (Payne-Hanek reduction)
    T = int(mp.floor(2 / mp.pi * mp.mpf(2) ** 192))
    for k, w in enumerate(((T >> 128) & (2 ** 64 - 1), (T >> 64) & (2 ** 64 - 1), T & (2 ** 64 - 1))):
        out.append("#define AG_2OPI_W%d 0x%016xull" % (k, w))
    out.append("#define AG_SC_TAB_OFF 1664")
    out.append("__device__ __align__(16) const float kSinCos2048[%d] = {%s};" % (len(packed), ", ".join(fl(v) for v in packed)))
    # pi/2 in three parts: the first with 12 bits so k*P1 is exact for |k| < 2^12.
    pio2 = mp.pi / 2
    p1 = trunc_bits(pio2, 12)
    p2 = trunc_bits(pio2 - p1, 24)
    p3 = f32(pio2 - p1 - p2)
    out.append("#define AG_PIO2_1 %s" % fl(p1))
    out.append("#define AG_PIO2_2 %s" % fl(p2))
    out.append("#define AG_PIO2_3 %s" % fl(p3))
    out.append("#define AG_TWO_OVER_PI %s" % fl(2 / mp.pi))
    pih, pil = split2(mp.pi)
    out.append("#define AG_PI_HI %s" % fl(pih))
    ph2, pl2 = split2(mp.pi / 2)
    out.append("#define AG_PIO2_HI %s" % fl(ph2))
    out.append("#define AG_PIO2_LO %s" % fl(pl2))
    out.append("#define AG_PI_LO %s" % fl(pil))
    out += ["}  // namespace e64", "}  // namespace ag", ""]
    with open(os.path.join(HERE, "ag_emu64_tables.cuh"), "w") as f:
        f.write("\n".join(out))

    # The Box-Muller sine: sin(pi k/4096) and pi cos(pi k/4096) over the whole
    # period, k in [0, 8192], packed (S hi, S lo, pi C hi, pi C lo). The angle
    # pi v is reduced in integers to one of these points and an exact remainder
    # t of at most 2^-13 half-turns, with no quadrant step; the factor pi of
    # the remainder's leading term rides on the table (C pi t = (pi C) t).
    # Included only by plans that draw normals.
    packed = []
    for k in range(0, 8193):
        a = mp.pi * mp.mpf(k) / 4096
        packed += list(split2(mp.sin(a))) + list(split2(mp.pi * mp.cos(a)))
    bm = ["// generated by gen_emu64_tables.py -- do not edit", "#pragma once", "namespace ag {", "namespace e64 {",
          "__device__ __align__(16) const float kSinCosPiPeriod[%d] = {%s};" % (len(packed), ", ".join(fl(v) for v in packed)),
          "}  // namespace e64", "}  // namespace ag", ""]
    with open(os.path.join(HERE, "ag_emu64_bm_tables.cuh"), "w") as f:
        f.write("\n".join(bm))


if __name__ == "__main__":
    main()
