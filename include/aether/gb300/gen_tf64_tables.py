"""Generate ag_tf64_tables.cuh and ag_tf64_trig_tables.cuh: the tables and split constants of the
triple-float (three floats, about 72 significant bits) function kernels in
ag_tf64.cuh: the logarithm's, the exponential's (2^(j/64) and ln2/64, Tang
1989) and the sine's and cosine's (pi/2 in four parts for a Cody-Waite
reduction, sin and cos of j/2048).

Every value is computed here with mpmath at 200 bits and split three ways
(x = fl(v), y = fl(v - x), z = fl(v - x - y)). The logarithm keeps the
reduction points c_i of the double-float tables (ag_emu64_tables.cuh, the same
formula), so one index computation serves both; only -log c_i and e ln2 gain
their third float here.

usage: python include/aether/gb300/gen_tf64_tables.py
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
    return hi, f32(mp.mpf(v) - hi)


def split3(v):
    x = f32(v)
    y = f32(mp.mpf(v) - x)
    z = f32(mp.mpf(v) - x - y)
    return x, y, z


def fl(x):
    s = np.float32(x)
    r = repr(float(s))
    if "inf" in r or "nan" in r:
        raise ValueError(r)
    return "%sf" % np.format_float_scientific(s, precision=9, unique=False)


def main():
    out = ["// generated by gen_tf64_tables.py -- do not edit", "#pragma once", "namespace ag {", "namespace t64 {"]

    # --- log: the reduction points of the double-float tables, i in [-256, 512]
    # packed (c_i, -log c_i as three floats): one 16-byte load per lookup
    packed = []
    for i in range(-256, 513):
        c = 1.0 if i == 0 else f32(1 / (1 + mp.mpf(i) / 1024))
        packed += [c] + list(split3(-mp.log(mp.mpf(c))))
    out.append("#define AG_TF_LOG_TAB_OFF 256")
    out.append("__device__ __align__(16) const float kLogCL3[%d] = {%s};" % (len(packed), ", ".join(fl(v) for v in packed)))
    # e ln2 for every exponent the reduction can produce, e in [-129, 130],
    # packed (three floats, 0)
    packed = []
    for e in range(-129, 131):
        packed += list(split3(e * mp.log(2))) + [0.0]
    out.append("#define AG_TF_LN2_TAB_OFF 129")
    out.append("__device__ __align__(16) const float kLn2Mul3[%d] = {%s};" % (len(packed), ", ".join(fl(v) for v in packed)))
    # 1/3 as a float pair: the one coefficient of the log1p series that must
    # carry more than a float's precision (its product with t sits 2^-12 below
    # the series' leading 1/2)
    h, l = split2(mp.mpf(1) / 3)
    out.append("#define AG_TF_THIRD_HI %s" % fl(h))
    out.append("#define AG_TF_THIRD_LO %s" % fl(l))
    # --- exp: 2^(j/64), j in [0, 63], packed (three floats, 0) ---------------
    packed = []
    for j in range(64):
        packed += list(split3(mp.power(2, mp.mpf(j) / 64))) + [0.0]
    out.append("__device__ __align__(16) const float kExp2Tab3[%d] = {%s};" % (len(packed), ", ".join(fl(v) for v in packed)))
    x, y, z = split3(mp.log(2) / 64)
    out.append("#define AG_TF_LN2_64_X %s" % fl(x))
    out.append("#define AG_TF_LN2_64_Y %s" % fl(y))
    out.append("#define AG_TF_LN2_64_Z %s" % fl(z))
    out.append("#define AG_TF_INV_LN2_64 %s" % fl(64 / mp.log(2)))
    for name, v in (("SIXTH", mp.mpf(1) / 6), ("24TH", mp.mpf(1) / 24)):
        h, l = split2(v)
        out.append("#define AG_TF_%s_HI %s" % (name, fl(h)))
        out.append("#define AG_TF_%s_LO %s" % (name, fl(l)))

    out += ["}  // namespace t64", "}  // namespace ag", ""]
    with open(os.path.join(HERE, "ag_tf64_tables.cuh"), "w") as f:
        f.write("\n".join(out))

    # The sine's and cosine's tables, in their own header: only plans with
    # trigonometric nodes include them.
    out = ["// generated by gen_tf64_tables.py -- do not edit", "#pragma once", "namespace ag {", "namespace t64 {"]
    # --- sin/cos: pi/2 in four parts, the first with 14 significant bits so q
    # times it is exact for |q| < 2^10; sin and cos of j/2048 for j in
    # [-1664, 1664] as three floats each, packed (S x, y, z, C x), (C y, z, 0, 0)
    pio2 = mp.pi / 2
    e = mp.floor(mp.log(pio2, 2))
    p0 = f32(mp.floor(pio2 * mp.mpf(2) ** (13 - e)) / mp.mpf(2) ** (13 - e))
    p1 = f32(pio2 - p0)
    p2 = f32(pio2 - p0 - p1)
    p3 = f32(pio2 - p0 - p1 - p2)
    for k, v in enumerate((p0, p1, p2, p3)):
        out.append("#define AG_TF_PIO2_%d %s" % (k, fl(v)))
    out.append("#define AG_TF_2OPI %s" % fl(2 / mp.pi))
    packed = []
    for j in range(-1664, 1665):
        a = mp.mpf(j) / 2048
        S, C = split3(mp.sin(a)), split3(mp.cos(a))
        packed += [S[0], S[1], S[2], C[0], C[1], C[2], 0.0, 0.0]
    out.append("#define AG_TF_SC_TAB_OFF 1664")
    out.append("__device__ __align__(16) const float kSinCos3[%d] = {%s};" % (len(packed), ", ".join(fl(v) for v in packed)))
    out += ["}  // namespace t64", "}  // namespace ag", ""]
    with open(os.path.join(HERE, "ag_tf64_trig_tables.cuh"), "w") as f:
        f.write("\n".join(out))


if __name__ == "__main__":
    main()
