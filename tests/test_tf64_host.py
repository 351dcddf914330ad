"""Host check of the FP64-grade triple-float kernels (ag_tf64.cuh) against
113-bit arithmetic (tests/emu_host/tf_check.cpp, __float128): the split is
exact and reassembles to the same double; sums, products, quotients, square
roots, reciprocal square roots, logarithms, log1p, exp, sin and cos stay within
a small fraction of a double ulp (sin and cos also near multiples of pi/2); the large streaming expression
sqrt(a*a+b*b)*log1p(|c|) + rsqrt(1+d0*d0) rounds to within
FP64_GRADE_EXACT_ULPS of its term scale."""

import json
import os
import shutil
import subprocess

import pytest

from aether_gb300.accuracy import FP64_GRADE_EXACT_ULPS

HERE = os.path.dirname(os.path.abspath(__file__))

# units of 2^-53 of the result (of the larger operand for sums)
BOUNDS = {"split": 0.0, "add": 0.01, "sub": 0.01, "mul": 0.01, "div": 0.01, "sqr_then_mul": 0.01, "cancel": 0.01,
          "sqrt": 0.01, "rsqrt": 0.01, "recip": 0.01, "log": 0.25, "log_near_1": 0.25, "log1p": 0.25,
          "log1p_nn": 0.25, "log1p_neg": 0.25, "exp": 0.25, "exp_small": 0.25, "sin": 0.25, "cos": 0.25,
          "sin_unit": 0.25, "trig_near_multiples": 0.5}


@pytest.fixture(scope="module")
def report(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("tf") / "tf_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-o", exe,
                        os.path.join(HERE, "emu_host", "tf_check.cpp"), "-lquadmath"], capture_output=True, text=True)
    if r.returncode != 0 and "quadmath" in r.stderr:
        pytest.skip("no libquadmath")
    assert r.returncode == 0, r.stderr
    return json.loads(subprocess.check_output([exe]))


@pytest.mark.parametrize("name", sorted(BOUNDS))
def test_operation_error(report, name):
    s = report[name]
    assert s["n"] > 100000 and s["bad"] == 0, s
    assert s["max"] <= BOUNDS[name], s


def test_expression_rounds_once(report):
    s = report["expr_term_ulps"]
    assert s["n"] > 100000
    assert s["max"] <= FP64_GRADE_EXACT_ULPS, s
    assert s["mean"] < 0.5, s
