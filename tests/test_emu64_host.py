"""The double-float kernels of the emulated FP64 mode (ag_emu64.cuh), built as
host C++ through tests/emu_host/host_shim.h and checked against long double.
Errors are in units of 2^-53 relative (double ulps at the bottom of a binade).
A double enters as a truncated 24-bit head and a rounded float tail, up to
2^-47 = 64 units off; a product of two such inputs is therefore bounded by
about 2 x 64 plus its own rounding, hence the mul bound of 320; a quotient
(one Newton correction on a float reciprocal) adds a few such roundings of
terms up to 2^-23 of the quotient, hence 384 for div and recip.

Bounds hold for well-conditioned uses; where a function is ill-conditioned
with respect to a relative perturbation of its input (log near 1, exp at large
|x|, sums that cancel), the error is the 2^-48 input rounding of a
double-float times that condition number, and the GPU tests check those
expressions against the magnitude of their terms."""

import json
import os
import subprocess

import pytest

from conftest import REPO

BOUNDS = {
    "roundtrip": 33, "sqrt": 256, "rsqrt": 320, "exp_small": 128, "log1p": 160, "log1p_tiny": 256,
    "log1p_neg": 1024, "sin": 160, "cos": 160, "recip": 384, "mul": 320, "div": 384, "cfg2a": 256, "cfg2a_gen": 256,
    "cfg1_termscale": 256, "normal_abs_rel": 256, "trig_large_f32": 256,
    # 2^22 draws each: the long tails (the stated bounds of the emulated mode)
    "cfg2a_gen_2p22": 512, "normal_2p22": 256,
}


@pytest.fixture(scope="module")
def emu_report(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("emu") / "emu_check")
    src = os.path.join(REPO, "tests", "emu_host", "emu_check.cpp")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-o", exe, src])
    return json.loads(subprocess.check_output([exe]))


@pytest.mark.parametrize("name", sorted(BOUNDS))
def test_emulated_function_error_bounds(emu_report, name):
    r = emu_report[name]
    assert r["n"] > 100000 and r["bad"] == 0
    assert r["max"] <= BOUNDS[name], (name, r)


def test_normals_inside_the_reference_tolerance(emu_report):
    # random/detail/Backend.h:44-51: abs+rel 1e-12 for double normals.
    assert emu_report["normal_abs_rel"]["max"] * 2.0 ** -53 < 1e-12
