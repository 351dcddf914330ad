"""The stated error bounds of each lowering, in one place.

Every check of a result against the FP64 oracle -- the GPU tests, smoke()
and the benchmark's check of its own run -- reads its bound from here, in the
units named beside it.

Units:
  term scale  the largest magnitude among an expression's additive terms at a
              sample (for d = sqrt(a*a+b*b)*log1p(|c|) + rsqrt(1+d0*d0):
              max(|sqrt(a*a+b*b)*log1p(|c|)|, |rsqrt(1+d0*d0)|)), so that a
              cancellation between terms does not inflate a relative error;
  2^-53       of that scale: err = |got - ref| / scale / 2^-53;
  abs+rel     for normals, the reference's form |got - ref| / (1 + |ref|)
              (random/detail/Backend.h:44-51), in units of 2^-53.

The reference's own contracts these are read against: device FP64 sin/cos
within 2 ulp (math/detail/BoundedTrig.h:31-37); Philox normals within 1e-12
abs+rel of cuRAND's (tests/random/golden_random.h:437-441), which is about
9007 x 2^-53.
"""

# Native FP64 lowering (math 0): CUDA's FP64 functions. Arithmetic and
# geometry are bit-exact with contraction off; a transcendental expression
# stays within this many ulp of its largest term (spacing of the term scale).
NATIVE_EXPR_ULPS = 4
# Native Box-Muller normals (CUDA's FP64 log, sqrt and sin), abs+rel in 2^-53.
NATIVE_NORMAL_BOUND_2M53 = 8

# Emulated FP64 lowering (math 1): double-float arithmetic on the FP32/INT
# pipes. Inputs enter as a float pair (at most 2^-47 off), so the error is
# that rounding times the expression's condition number plus the double-float
# evaluation's own: measured 316 x 2^-53 of the term scale over 2^25 samples
# of the large streaming expression, 178 for the plain config-1 expression.
EMU_EXPR_BOUND_2M53 = 512
# Emulated Box-Muller normals, abs+rel (measured 194 x 2^-53 over 2^25 draws).
EMU_NORMAL_BOUND_2M53 = 256

# FP64-grade lowering (math 3): doubles split exactly into three floats; sums,
# products, quotients, sqrt, rsqrt, log, log1p, exp, sin and cos in
# triple-float arithmetic (each within about 2^-60 relative on the host check
# against 113-bit arithmetic, tests/emu_host/tf_check.cpp), the other
# functions on the native pipe;
# each output is the triple-float value rounded once to a double. Against
# exact arithmetic: this many ulps of the term scale (measured 1.0 on the
# host, the final rounding). Against the oracle (itself a few ulps from exact)
# the native bound NATIVE_EXPR_ULPS applies.
FP64_GRADE_EXACT_ULPS = 2

# Precision form (math 2): float-float outputs and the FP64-finished global
# sum, relative to FP64 evaluation of the same f32 inputs.
PRECISION_FF_REL = 1e-12


def term_scale_error_2m53(got, ref, scale):
    """max |got - ref| / scale in units of 2^-53 (numpy arrays)."""
    import numpy as np
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    err = np.where(same, 0.0, np.abs(got - ref) / np.abs(np.asarray(scale, dtype=np.float64)))
    return float(np.max(err)) / 2.0 ** -53 if err.size else 0.0


def term_scale_error_ulp(got, ref, scale):
    """max |got - ref| / spacing(max(|ref|, scale)): ulps of the largest term."""
    import numpy as np
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    mag = np.maximum(np.abs(ref), np.abs(np.asarray(scale, dtype=np.float64)))
    err = np.where(same, 0.0, np.abs(got - ref) / np.spacing(mag))
    return float(np.max(err)) if err.size else 0.0


def abs_rel_error_2m53(got, ref):
    """max |got - ref| / (1 + |ref|) in units of 2^-53 (numpy arrays)."""
    import numpy as np
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.max(np.abs(got - ref) / (1.0 + np.abs(ref)))) / 2.0 ** -53 if ref.size else 0.0
