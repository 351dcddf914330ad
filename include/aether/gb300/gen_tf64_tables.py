"""Generate ag_tf64_tables.cuh: the tables and split constants of the
triple-float (three floats, about 72 significant bits) function kernels in
ag_tf64.cuh.

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
    out += ["}  // namespace t64", "}  // namespace ag", ""]
    with open(os.path.join(HERE, "ag_tf64_tables.cuh"), "w") as f:
        f.write("\n".join(out))


if __name__ == "__main__":
    main()
