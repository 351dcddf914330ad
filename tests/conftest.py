import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
ORACLE = os.path.join(REPO, "oracle")
if ORACLE not in sys.path:
    sys.path.insert(0, ORACLE)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def ref_cases():
    return np.load(os.path.join(GOLDEN, "ref_cases.npz"))


@pytest.fixture(scope="session")
def philox_golden():
    import json
    with open(os.path.join(GOLDEN, "philox_golden.json")) as f:
        return json.load(f)


def ulp_diff(a, b):
    """Distance in units in the last place between same-typed float arrays
    (NaN == NaN, +0 == -0)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype == np.float64:
        ia = a.view(np.int64).astype(np.int64)
        ib = b.view(np.int64).astype(np.int64)
        big = np.int64(0x7FFFFFFFFFFFFFFF)
    else:
        ia = a.view(np.int32).astype(np.int64)
        ib = b.view(np.int32).astype(np.int64)
        big = np.int64(0x7FFFFFFF)
    ia = np.where(ia < 0, -(ia & big), ia)
    ib = np.where(ib < 0, -(ib & big), ib)
    d = np.abs(ia - ib).astype(np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    d[both_nan] = 0
    d[np.isnan(a) ^ np.isnan(b)] = np.inf
    return d


def assert_ulp(got, ref, ulps, scale=None, what=""):
    """|got - ref| <= ulps * spacing(max(|ref|, scale)): an ulp bound on the
    result, measured against the magnitude of the largest term when a
    cancellation makes the result itself small."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    mag = np.abs(ref) if scale is None else np.maximum(np.abs(ref), np.abs(scale))
    err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    bound = ulps * np.spacing(mag.astype(ref.dtype)).astype(np.float64)
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    bad = ~same & ~(err <= bound)
    if bad.any():
        i = np.argwhere(bad)[0]
        raise AssertionError("%s: %d values beyond %g ulp; first at %s: got %r ref %r (err %g, bound %g)"
                             % (what, bad.sum(), ulps, tuple(i), got[tuple(i)], ref[tuple(i)], err[tuple(i)],
                                bound[tuple(i)]))


def assert_term_scale(got, ref, bound_2m53, scale, what=""):
    """|got - ref| <= bound_2m53 * 2^-53 * scale, scale the largest term's
    magnitude (the unit of aether_gb300.accuracy's emulated bounds)."""
    from aether_gb300.accuracy import term_scale_error_2m53
    e = term_scale_error_2m53(got, ref, scale)
    assert e <= bound_2m53, "%s: %.1f x 2^-53 of the term scale, bound %d" % (what, e, bound_2m53)
