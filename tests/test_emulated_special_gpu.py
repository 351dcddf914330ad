"""Emulated-FP64 elementwise functions on special and extreme inputs: NaN,
+-Inf, zeros, subnormals, huge values, and trig arguments in the integer
Payne-Hanek range (6000..2^24) and beyond it. Samples outside the
double-float input range [2^-50, 2^60] equal the native kernel bit for bit
(the per-lane native recomputation); in-range samples stay within the input-rounding error model
(a double enters as 2^-48-accurate head and tail, so an argument x carries an
absolute uncertainty of about 2^-48 |x|)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


import aether_gb300 as ag

SPECIAL = [0.0, -0.0, 5e-324, -1e-310, 1e-30, -1e-18, 2.0 ** -61, 0.5, -0.75, 1.0, 3.0, -2.5, 7.0, 100.0,
           -700.0, 709.5, 6000.0, -6001.5, 1e5, -123456.789, 2.0 ** 23 + 0.5, 2.0 ** 24 - 1.0, 2.0 ** 24,
           -3e7, 1e15, 2.0 ** 61, 1e30, 1e200, np.inf, -np.inf, np.nan]


def _run(fn, x):
    n = x.size
    a = ag.Array("f64", (1,), n)
    a.upload(x.reshape(1, n))
    out = {}
    for m in (0, 1):
        d = ag.Array("f64", (1,), n)
        ag.assign(d, fn(a.view()), math=m)
        out[m] = d.host()[0]
    return out[1], out[0]


@pytest.mark.parametrize("name", ["sin", "cos", "exp", "log", "log1p", "sqrt", "rsqrt", "hypot_sq"])
def test_emulated_functions_on_special_inputs(name):
    rng = np.random.default_rng(11)
    base = np.array(SPECIAL, dtype=np.float64)
    wide = np.concatenate([base, rng.uniform(-2.0 ** 24, 2.0 ** 24, 4000), rng.uniform(-40, 40, 4000)])
    if name in ("log", "log1p", "sqrt", "rsqrt"):
        wide = np.concatenate([wide, np.abs(wide)])
    fn = {"sin": ag.cwiseSin, "cos": ag.cwiseCos, "exp": ag.cwiseExp, "log": ag.cwiseLog,
          "log1p": ag.cwiseLog1p, "sqrt": ag.cwiseSqrt, "rsqrt": ag.cwiseRsqrt,
          # sqrt of a sum of squares: the non-negative form (zero, no sign test)
          "hypot_sq": lambda v: ag.cwiseSqrt(v * v + v * v)}[name]
    emu, nat = _run(fn, wide)
    # NaN exactly where the native kernel gives NaN (negative arguments of
    # sqrt/rsqrt/log included: those lanes take the native path)
    assert np.array_equal(np.isnan(emu), np.isnan(nat))
    ax = np.abs(wide)
    inrange = (ax >= 2.0 ** -50) & (ax <= 2.0 ** 60)
    if name in ("sin", "cos"):
        inrange &= ax < 2.0 ** 24
    # outside the range: the native result, bit for bit (NaN for NaN)
    assert np.array_equal(emu[~inrange], nat[~inrange], equal_nan=True)
    ok = inrange & np.isfinite(nat) & (np.abs(nat) > 2.0 ** -90) & (np.abs(nat) < 2.0 ** 126)
    e, r, x = emu[ok], nat[ok], wide[ok]
    if name in ("sin", "cos"):
        tol = 2.0 ** -45 * np.maximum(1.0, np.abs(x))
    elif name in ("sqrt", "rsqrt", "hypot_sq"):
        tol = 2.0 ** -45 * np.abs(r)
    elif name == "exp":
        tol = 2.0 ** -45 * np.abs(r) * np.maximum(1.0, np.abs(x))
    else:
        tol = 2.0 ** -46 * (1.0 + np.abs(r))
    bad = np.abs(e - r) > tol
    assert not bad.any(), (name, x[bad][:5], e[bad][:5], r[bad][:5])
    # everything the emulated kernel produced for in-range inputs is finite
    # where the native result is
    assert np.all(np.isfinite(emu[inrange & np.isfinite(nat)]))


def test_precision_form_trig_on_special_float_inputs():
    """FP32 storage: trig of NaN/Inf and of floats past 2^24 takes the native
    lane; floats below it reduce in integers."""
    x = np.array([0.0, 1e-30, 6000.0, 1e5, 2.0 ** 24 - 1, 2.0 ** 24, 3e7, 1e30, np.inf, -np.inf, np.nan,
                  -12345.678], dtype=np.float32)
    n = x.size
    a = ag.Array("f32", (1,), n)
    a.upload(x.reshape(1, n))
    d = ag.Array("ff", (1,), n)
    ag.assign(d, ag.cwiseSin(a.view()), math=2)
    got = d.host_ff()[0]
    with np.errstate(invalid="ignore"):
        ref = np.sin(x.astype(np.float64))
    fin = np.isfinite(ref)
    assert np.all(np.isnan(got[~fin]))
    assert np.all(np.abs(got[fin] - ref[fin]) <= 1e-12 * np.maximum(1.0, np.abs(ref[fin])))


def test_precision_form_f32_output_on_special_inputs():
    """FP32 storage and an f32 destination: lanes outside the double-float
    range are recomputed natively after the stores and rounded once to f32,
    like the in-range lanes."""
    x = np.array([0.0, 1e-30, 0.5, -3.0, 6000.0, 1e5, 2.0 ** 24, 3e7, 1e30, np.inf, -np.inf, np.nan,
                  -12345.678, 1e-40], dtype=np.float32)
    x = np.concatenate([x, np.random.default_rng(3).uniform(-50, 50, 997).astype(np.float32)])
    n = x.size
    a = ag.Array("f32", (1,), n)
    a.upload(x.reshape(1, n))
    d = ag.Array("f32", (1,), n)
    ag.assign(d, ag.cwiseSin(a.view()) * ag.cwiseSqrt(ag.cwiseAbs(a.view())), math=2)
    got = d.host()[0]
    with np.errstate(invalid="ignore", over="ignore"):
        ref = (np.sin(x.astype(np.float64)) * np.sqrt(np.abs(x.astype(np.float64))))
    fin = np.isfinite(ref)
    assert np.array_equal(np.isnan(got), np.isnan(ref.astype(np.float32)))
    # one f32 rounding of a value within 1e-12 of the FP64 one
    r32 = ref[fin].astype(np.float32)
    assert np.all(np.abs(got[fin].astype(np.float64) - r32.astype(np.float64))
                  <= np.spacing(np.abs(r32)).astype(np.float64))


def test_tiny_intermediate_products_take_the_native_path():
    """A product below 2^-102 would leave the pair's error terms subnormal:
    such lanes are flagged and recomputed natively, so a tiny intermediate
    scaled back up keeps FP64 accuracy."""
    rng = np.random.default_rng(5)
    n = 4096
    xs = [np.exp2(rng.uniform(-49.9, -30, n)) * rng.choice([-1.0, 1.0], n) for _ in range(3)]
    arrs = []
    for x in xs:
        a = ag.Array("f64", (1,), n)
        a.upload(x.reshape(1, n))
        arrs.append(a)
    a, b, c = (x.view() for x in arrs)
    out = {}
    for m in (0, 1):
        d = ag.Array("f64", (1,), n)
        ag.assign(d, ((a * b) * c) * 2.0 ** 100, math=m)
        out[m] = d.host()[0]
    emu, nat = out[1], out[0]
    assert np.all(np.abs(emu - nat) <= 2.0 ** -45 * np.abs(nat))
