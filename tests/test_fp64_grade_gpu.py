"""GPU parity of the FP64-grade lowering (math = 3, ag_tf64.cuh): f64 plans
evaluated in triple-float arithmetic on the FP32/INT pipes.

Bounds (aether_gb300.accuracy): against exact arithmetic (long double, at
least 64 significant bits) FP64_GRADE_EXACT_ULPS ulps of the term scale;
against the oracle and the reference's own outputs (double arithmetic, a few
ulps from exact themselves) the native bound NATIVE_EXPR_ULPS. Samples outside
the triple-float range take the native FP64 kernel bit for bit; Philox fills
are bit-exact (uniforms exactly representable, normals from the native draw).
"""

import numpy as np
import pytest

from conftest import assert_ulp

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


import aether_gb300 as ag
from aether_gb300.accuracy import FP64_GRADE_EXACT_ULPS, NATIVE_EXPR_ULPS


def dev_array(host):
    host = np.asarray(host)
    if host.ndim == 1:
        host = host[None, :]
    arr = ag.Array("f64", (host.shape[0],), host.shape[1])
    arr.upload(host)
    return arr


def _cfg2a(a, b, c, d0):
    return ag.cwiseSqrt(a * a + b * b) * ag.cwiseLog1p(ag.cwiseAbs(c)) + ag.cwiseRsqrt(ag.constant(1.0, (3,)) + d0 * d0)


def _cfg1(a, b, c):
    return a + b * c + ag.cwiseSin(a) * ag.cwiseExp((c * c) * (-1.0))


def _cfg2a_exact(A, B, C, D0):
    L = [np.asarray(x, dtype=np.longdouble) for x in (A, B, C, D0)]
    a, b, c, d0 = L
    t1 = np.sqrt(a * a + b * b) * np.log1p(np.abs(c))
    t2 = 1 / np.sqrt(1 + d0 * d0)
    return t1 + t2, np.maximum(np.abs(t1), np.abs(t2))


def _ulps_of_scale(got, exact, scale):
    """max |got - exact| in ulps of max(|exact|, term scale): the result's own
    rounding is half an ulp of the result, which can exceed the term scale
    when terms of one sign add up."""
    mag = np.maximum(np.abs(np.asarray(exact, dtype=np.float64)), np.asarray(scale, dtype=np.float64))
    sp = np.spacing(mag)
    return float(np.max(np.abs(np.asarray(got, dtype=np.longdouble) - exact) / sp.astype(np.longdouble)))


def test_config2a_against_reference_and_exact(ref_cases):
    z = ref_cases
    cols = [z[k] for k in ("cfg2a_a", "cfg2a_b", "cfg2a_c", "cfg2a_d0")]
    ins = [dev_array(x) for x in cols]
    d = ag.Array("f64", (3,), 1000)
    ag.assign(d, _cfg2a(*(x.view() for x in ins)), math=3)
    exact, scale = _cfg2a_exact(*cols)
    assert_ulp(d.host(), z["cfg2a_d"], NATIVE_EXPR_ULPS, scale.astype(np.float64), "config 2a FP64-grade vs reference")
    assert _ulps_of_scale(d.host(), exact, scale) <= FP64_GRADE_EXACT_ULPS


def test_config2a_full_size_subsample(oracle):
    n = 1 << 24
    arrs = [ag.Array("f64", (3,), n) for _ in range(4)]
    for k, arr in enumerate(arrs):
        ag.assign(arr, ag.Generator(7).substream(k).uniform(3, -4.0, 4.0), math=3)
    d = ag.Array("f64", (3,), n)
    ag.assign(d, _cfg2a(*(x.view() for x in arrs)), math=3)
    idx = torch.randint(0, n, (1 << 15,), generator=torch.Generator().manual_seed(3)).cuda()
    sub = [np.ascontiguousarray(x.data[:, idx].cpu().numpy()) for x in arrs]
    got = d.data[:, idx].cpu().numpy()
    exact, scale = _cfg2a_exact(*sub)
    assert_ulp(got, oracle.cfg2a(*sub), NATIVE_EXPR_ULPS, scale.astype(np.float64), "config 2a FP64-grade, 2^24")
    assert _ulps_of_scale(got, exact, scale) <= FP64_GRADE_EXACT_ULPS


def test_config1_against_reference(ref_cases):
    z = ref_cases
    a, b, c = (dev_array(z[k]) for k in ("cfg1_a", "cfg1_b", "cfg1_c"))
    d = ag.Array("f64", (3,), 1000)
    ag.assign(d, _cfg1(a.view(), b.view(), c.view()), math=3)
    A, B, C = z["cfg1_a"], z["cfg1_b"], z["cfg1_c"]
    scale = np.maximum.reduce([np.abs(A), np.abs(B * C), np.abs(np.sin(A) * np.exp(-C * C))])
    assert_ulp(d.host(), z["cfg1_d"], NATIVE_EXPR_ULPS, scale, "config 1 FP64-grade vs reference")


def test_config1_full_size_against_exact(oracle):
    """Config 1 at 2^20 samples: sin and exp in triple-float as well."""
    n = 1 << 20
    arrs = [ag.Array("f64", (3,), n) for _ in range(3)]
    for k, arr in enumerate(arrs):
        ag.assign(arr, ag.Generator(42).substream(k).uniform(3, -1.0, 1.0))
    d = ag.Array("f64", (3,), n)
    ag.assign(d, _cfg1(*(x.view() for x in arrs)), math=3)
    A, B, C = (np.asarray(x.host(), dtype=np.longdouble) for x in arrs)
    t3 = np.sin(A) * np.exp(-C * C)
    exact = A + B * C + t3
    scale = np.maximum.reduce([np.abs(A), np.abs(B * C), np.abs(t3)])
    assert _ulps_of_scale(d.host(), exact, scale) <= FP64_GRADE_EXACT_ULPS
    assert_ulp(d.host(), oracle.cfg1(*(x.host() for x in arrs)), NATIVE_EXPR_ULPS, scale.astype(np.float64),
               "config 1 FP64-grade vs oracle")


@pytest.mark.parametrize("fn", ["exp", "sin", "cos"])
def test_functions_against_exact(fn):
    """exp over (-50, 80), sin and cos over |x| < 1000 (the triple-float
    ranges; lanes outside them or near nonzero multiples of pi/2 are native)."""
    n = 1 << 16
    x = ag.Array("f64", (1,), n)
    lo, hi = (-50.0, 80.0) if fn == "exp" else (-1000.0, 1000.0)
    ag.assign(x, ag.Generator(29).uniform(1, lo, hi))
    X = x.view()
    e = {"exp": ag.cwiseExp(X), "sin": ag.cwiseSin(X), "cos": ag.cwiseCos(X)}[fn]
    d = ag.Array("f64", (1,), n)
    ag.assign(d, e, math=3)
    H = np.asarray(x.host(), dtype=np.longdouble)
    exact = {"exp": np.exp, "sin": np.sin, "cos": np.cos}[fn](H)
    err = np.abs(np.asarray(d.host(), dtype=np.longdouble) - exact) / np.spacing(np.abs(exact.astype(np.float64)))
    assert float(err.max()) <= 1.0, (fn, float(err.max()))


def _q(x):
    return np.asarray(x, dtype=np.longdouble)


@pytest.mark.parametrize("name", ["cross", "qrot", "div_mix", "log_mix"])
def test_nodes_against_exact(name):
    """Geometry, quotients and logarithms against long-double evaluation of
    the same formula, in ulps of each sample's term scale (the largest
    magnitude among the terms its sums combine)."""
    n = 8192
    g = ag.Generator(19)
    a, b, q = ag.Array("f64", (3,), n), ag.Array("f64", (3,), n), ag.Array("f64", (4,), n)
    ag.assign(a, g.substream(0).uniform(3, -2.0, 2.0))
    ag.assign(b, g.substream(1).uniform(3, 0.5, 3.0))
    ag.assign(q, g.substream(2).uniform(4, -1.0, 1.0))
    A, B, Q = a.view(), b.view(), q.view()
    HA, HB, HQ = _q(a.host()), _q(b.host()), _q(q.host())
    if name == "cross":
        e = A.cross(B)
        terms = [HA[1] * HB[2], HA[2] * HB[1], HA[2] * HB[0], HA[0] * HB[2], HA[0] * HB[1], HA[1] * HB[0]]
        exact = np.stack([terms[0] - terms[1], terms[2] - terms[3], terms[4] - terms[5]])
        scale = np.stack([np.maximum(abs(terms[0]), abs(terms[1])), np.maximum(abs(terms[2]), abs(terms[3])),
                          np.maximum(abs(terms[4]), abs(terms[5]))])
    elif name == "qrot":
        e = Q.quatRotate(A)
        w, x, y, z = HQ
        # v' = v + 2 w (u x v) + 2 u x (u x v), u = (x, y, z)
        u = np.stack([x, y, z])
        uv = np.stack([u[1] * HA[2] - u[2] * HA[1], u[2] * HA[0] - u[0] * HA[2], u[0] * HA[1] - u[1] * HA[0]])
        uuv = np.stack([u[1] * uv[2] - u[2] * uv[1], u[2] * uv[0] - u[0] * uv[2], u[0] * uv[1] - u[1] * uv[0]])
        exact = HA + 2 * w * uv + 2 * uuv
        # every term is at most |v| (1 + 4 |q|^2) in magnitude
        scale = np.broadcast_to(np.sqrt((HA * HA).sum(axis=0)) * (1 + 4 * (w * w + x * x + y * y + z * z)), exact.shape)
    elif name == "div_mix":
        e = ag.cwiseDiv(A, B) + A * (1.0 / 3.0)
        exact = HA / HB + HA * _q(1.0 / 3.0)
        scale = np.maximum(abs(HA / HB), abs(HA) / 3)
    else:
        e = ag.cwiseLog(B) - ag.cwiseSqrt(B) * ag.cwiseRsqrt(B + A * A)
        t2 = np.sqrt(HB) / np.sqrt(HB + HA * HA)
        exact = np.log(HB) - t2
        scale = np.maximum(abs(np.log(HB)), abs(t2))
    d = ag.Array("f64", (3,), n)
    ag.assign(d, e, math=3)
    err = _ulps_of_scale(d.host(), exact, np.asarray(scale, dtype=np.float64))
    assert err <= FP64_GRADE_EXACT_ULPS, (name, err)


def test_guarded_inverse_against_native():
    n = 8192
    m = ag.Array("f64", (3, 3), n)
    ag.assign(m, ag.Generator(8).uniform(9, -1.0, 1.0).reshape((3, 3)))
    M = m.view()
    e = ag.select(ag.cwiseAbs(M.det()) > 1e-300, M.inverse(), ag.constant(0.0, (3, 3)))
    d3, d0 = ag.Array("f64", (3, 3), n), ag.Array("f64", (3, 3), n)
    ag.assign(d3, e, math=3)
    ag.assign(d0, e, math=0)
    got, nat = d3.host(), d0.host()
    H = m.host()
    keep = np.abs(np.linalg.det(H.T.reshape(n, 3, 3))) > 1e-2   # well-conditioned matrices
    scale = np.abs(nat[:, keep]).max(axis=0)
    assert np.all(np.abs(got[:, keep] - nat[:, keep]) <= 2.0 ** -40 * scale)


def test_fallback_reproduces_native_on_special_inputs():
    """Zeros, denormals, huge values, infinities and NaNs leave the
    triple-float range: those samples are the native kernel's bit for bit."""
    special = np.array([0.0, -0.0, 1e-310, -1e-200, 1e-30, 1e30, 1e200, np.inf, -np.inf, np.nan, 3.0, -2.5,
                        2.0 ** -41, 2.0 ** 61, 1e-11, 7.0], dtype=np.float64)
    rng = np.random.default_rng(5)
    # the specials mixed across the four operands, then samples with every
    # operand in range, so both sides of the range test occur
    cols = [np.concatenate([np.stack([rng.permutation(special) for _ in range(3)]),
                            rng.uniform(-4.0, 4.0, size=(3, 64))], axis=1) for _ in range(4)]
    n = cols[0].shape[1]
    ins = [dev_array(c) for c in cols]
    e = _cfg2a(*(x.view() for x in ins))
    d_nat, d_tf = ag.Array("f64", (3,), n), ag.Array("f64", (3,), n)
    ag.assign(d_nat, e, math=0, contract=1)
    ag.assign(d_tf, e, math=3)
    got, nat = d_tf.host(), d_nat.host()
    inrange = np.all([(np.abs(x) >= 2.0 ** -40) & (np.abs(x) <= 2.0 ** 60) for x in cols], axis=0)
    assert (~inrange).any() and inrange.any()
    assert np.array_equal(got[~inrange], nat[~inrange], equal_nan=True)
    with np.errstate(all="ignore"):
        exact, scale = _cfg2a_exact(*cols)
    assert _ulps_of_scale(got[inrange], exact[inrange], scale[inrange]) <= FP64_GRADE_EXACT_ULPS


def test_fills_are_exact(oracle):
    n = 100003
    a = ag.Array("f64", (3,), n)
    ag.assign(a, ag.Generator(7).substream(0).uniform(3, -4.0, 4.0), math=3)
    key = oracle.substream_key(oracle.generator_key(7), 0)
    assert np.array_equal(a.host(), oracle.fill_uniform_f64(key, -4.0, 4.0, 3, n))
    y3, y0 = ag.Array("f64", (1,), n), ag.Array("f64", (1,), n)
    ag.assign(y3, ag.Generator(7).substream(4).normal(1, 0.0, 1.0), math=3)
    ag.assign(y0, ag.Generator(7).substream(4).normal(1, 0.0, 1.0), math=0)
    assert np.array_equal(y3.host(), y0.host())


def test_scalars_and_literals_keep_their_bits():
    """A runtime scalar and a literal that need all 53 bits (1/3, pi) enter
    exactly: a * s - a * s is zero and (a + s) - s returns a."""
    n = 4096
    a = ag.Array("f64", (1,), n)
    ag.assign(a, ag.Generator(3).uniform(1, 1.0, 2.0))
    s = 1.0 / 3.0
    d = ag.Array("f64", (1,), n)
    ag.assign(d, (a.view() + s) - s, math=3)
    assert_ulp(d.host(), a.host(), 1, None, "(a + 1/3) - 1/3")
    ag.assign(d, a.view() * ag.literal(np.pi), math=3)
    ref = (a.host().astype(np.longdouble) * np.longdouble(np.pi))
    assert np.max(np.abs(d.host() - ref) / np.spacing(np.abs(d.host()))) <= 0.5 + 1e-6


def test_sum_and_accumulate():
    """Sum plans reduce the FP64-grade terms with the same compensated tree;
    += plans add them to the destination in FP64."""
    n = 1 << 20
    a = ag.Array("f64", (3,), n)
    ag.assign(a, ag.Generator(23).uniform(3, -2.0, 2.0))
    A = a.view()
    s3 = ag.global_sum(A.dot(A) + ag.cwiseLog1p(ag.cwiseAbs(A)).sum(), n, math=3).cpu().numpy()
    s0 = ag.global_sum(A.dot(A) + ag.cwiseLog1p(ag.cwiseAbs(A)).sum(), n, math=0).cpu().numpy()
    assert abs((s3[0] + s3[1]) - (s0[0] + s0[1])) <= 1e-13 * abs(s0[0])
    d3, d0 = ag.Array("f64", (3,), n), ag.Array("f64", (3,), n)
    ag.assign(d3, A * 0.5, math=0)
    ag.assign(d0, A * 0.5, math=0)
    e = ag.cwiseSqrt(ag.cwiseAbs(A)) + A * A
    for _ in range(2):
        ag.assign_add(d3, e, math=3)
        ag.assign_add(d0, e, math=0)
    H = a.host()
    scale = np.abs(H) * 0.5 + 2 * (np.sqrt(np.abs(H)) + H * H)
    assert_ulp(d3.host(), d0.host(), NATIVE_EXPR_ULPS, scale, "+= at FP64 grade")


@pytest.mark.parametrize("n", [1, 2, 31, 37, 255, 257, 513, 1025, 4099])
def test_ragged_sizes_and_tails(n):
    """Lane groups, chunk tails and single samples at FP64 grade: the
    deferred native recomputation and the stores stop at n."""
    arrs = [ag.Array("f64", (3,), n) for _ in range(4)]
    for k, arr in enumerate(arrs):
        ag.assign(arr, ag.Generator(40 + k).uniform(3, -4.0, 4.0))
    d = ag.Array("f64", (3,), n)
    d.data.fill_(7.0)
    ag.assign(d, _cfg2a(*(x.view() for x in arrs)), math=3)
    exact, scale = _cfg2a_exact(*(x.host() for x in arrs))
    assert _ulps_of_scale(d.host(), exact, scale) <= FP64_GRADE_EXACT_ULPS
    # capacity padding past n is left alone
    if d.data.shape[1] > n:
        assert bool((d.data[:, n:] == 7.0).all())


def test_misaligned_operands_take_the_scalar_kernel():
    n = 1001
    base = torch.zeros((3, 1100), dtype=torch.float64, device="cuda")
    a = ag.Array("f64", (3,), n)
    ag.assign(a, ag.Generator(5).uniform(3, -1.0, 1.0))
    base[:, 1:1 + n] = a.data[:, :n]
    mis = ag.expr.Operand(base.data_ptr() + 8, 1100, "f64", (3,))   # planes 8 bytes past 16
    d1, d2 = ag.Array("f64", (3,), n), ag.Array("f64", (3,), n)
    ag.assign(d1, ag.cwiseExp(a.view()) * ag.cwiseSqrt(a.view() * a.view() + 1.0), math=3)
    ag.assign(d2, ag.cwiseExp(mis) * ag.cwiseSqrt(mis * mis + 1.0), math=3)
    assert np.array_equal(d1.host(), d2.host())
