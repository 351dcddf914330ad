"""The precision form (math = 2): FP32 storage, float-float working values.

Inputs are FP32 with log-uniform magnitudes 10^U(-6,6) and random signs; the
FP64 oracle evaluates the same plans on the same FP32 values in double (the
global sum in long double). Bounds: float-float outputs and the global sum
within 1e-12 relative (the per-sample results relative to the magnitude of
their terms, the global sum relative to itself); outputs rounded to FP32
within 2^-23 relative to the magnitude of their terms."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


import aether_gb300 as ag


def loguniform_f32(seed, comps, n):
    """x = +-10^U(-6,6) in FP32, drawn on the device by the engine itself."""
    g = ag.Generator(seed)
    a = ag.Array("f32", (comps,), n)
    sign = g.substream(0).bernoulli(comps, 0.5) * 2.0 - 1.0
    mag = ag.cwiseExp(g.substream(1).uniform(comps, -6.0, 6.0) * 2.302585092994046)
    ag.assign(a, sign * mag)
    return a


def oracle_eval(oracle, expr, dst_dtype, shape, n, op="set", mode=1):
    ctx = ag.IrContext()
    ir = ag.expr.plan_text(dst_dtype, shape, op, expr, ctx)
    ops = [np.ascontiguousarray(owner.data.cpu().numpy()) for (_, _, _, _, owner) in ctx.operands]
    comps = int(np.prod(shape)) if shape else 1
    return oracle.eval_ir(ir, n, ops, scalars=ctx.scalars, keys=ctx.keys, dst_comps=comps, dst_dtype=np.float64,
                          mode=mode, reduce=op in ("sum", "setsum"))


@pytest.mark.parametrize("n", [1000, 1 << 20])
def test_dot8_and_global_sum_float_float(oracle, n):
    x = loguniform_f32(101, 8, n)
    y = loguniform_f32(202, 8, n)
    e = x.view().dot(y.view())
    d = ag.Array("ff", (1,), n)
    red = torch.zeros(2, dtype=torch.float64, device="cuda")
    ag.assign(d, e, op="setsum", reduce_out=red, math=2)
    got = d.host_ff()[0]
    ref, _ = oracle_eval(oracle, e, "f32", (), n, mode=1)
    ref = ref[0, :n]
    X, Y = x.host().astype(np.float64), y.host().astype(np.float64)
    scale = np.abs(X * Y).sum(axis=0)
    err = np.abs(got - ref) / scale
    assert err.max() <= 1e-12, err.max()
    # the global sum, relative to itself, against long double
    _, exact = oracle_eval(oracle, e, "f32", (), n, op="sum", mode=2)
    s = red.cpu().numpy()
    tot, ref_tot = s[0] + s[1], exact[0] + exact[1]
    assert abs(tot - ref_tot) <= 1e-12 * abs(ref_tot), (tot, ref_tot)


def test_dot8_rounded_to_f32(oracle):
    n = 100000
    x = loguniform_f32(5, 8, n)
    y = loguniform_f32(6, 8, n)
    e = x.view().dot(y.view())
    d = ag.Array("f32", (1,), n)
    ag.assign(d, e, math=2)
    ref, _ = oracle_eval(oracle, e, "f32", (), n, mode=1)
    X, Y = x.host().astype(np.float64), y.host().astype(np.float64)
    scale = np.abs(X * Y).sum(axis=0)
    err = np.abs(d.host()[0].astype(np.float64) - ref[0, :n]) / scale
    assert err.max() <= 2.0 ** -23, err.max()


def _p1(a, b, c):
    return a + b * c + ag.cwiseSin(a) * ag.cwiseExp((c * c) * (-1.0))


def _p2(a, b, c, d0):
    return ag.cwiseSqrt(a * a + b * b) * ag.cwiseLog1p(ag.cwiseAbs(c)) + ag.cwiseRsqrt(ag.constant(1.0, (3,)) + d0 * d0)


def test_p1_large_trig_arguments_float_float(oracle):
    """a up to +-1e5: the sine reduces in FP64 (the FP64 use the form allows)."""
    n = 1 << 18
    g = ag.Generator(77)
    a = ag.Array("f32", (3,), n)
    b = ag.Array("f32", (3,), n)
    c = ag.Array("f32", (3,), n)
    ag.assign(a, g.substream(0).uniform(3, -1e5, 1e5))
    ag.assign(b, g.substream(1).uniform(3, -1.0, 1.0))
    ag.assign(c, g.substream(2).uniform(3, -1.0, 1.0))
    e = _p1(a.view(), b.view(), c.view())
    d = ag.Array("ff", (3,), n)
    ag.assign(d, e, math=2)
    ref, _ = oracle_eval(oracle, e, "f32", (3,), n, mode=1)
    A, B, C = (v.host().astype(np.float64) for v in (a, b, c))
    scale = np.abs(A) + np.abs(B * C) + np.abs(np.exp(-C * C))
    err = np.abs(d.host_ff() - ref[:, :n]) / scale
    assert err.max() <= 1e-12, err.max()


def test_p2_float_float(oracle):
    n = 1 << 18
    ins = [loguniform_f32(300 + k, 3, n) for k in range(4)]
    e = _p2(*(v.view() for v in ins))
    d = ag.Array("ff", (3,), n)
    ag.assign(d, e, math=2)
    ref, _ = oracle_eval(oracle, e, "f32", (3,), n, mode=1)
    A, B, C, D0 = (v.host().astype(np.float64) for v in ins)
    scale = np.abs(np.sqrt(A * A + B * B) * np.log1p(np.abs(C))) + np.abs(1 / np.sqrt(1 + D0 * D0))
    err = np.abs(d.host_ff() - ref[:, :n]) / scale
    assert err.max() <= 1e-12, err.max()


def test_global_sum_is_deterministic_and_matches_f64_form(oracle):
    n = 1 << 20
    x = loguniform_f32(11, 8, n)
    y = loguniform_f32(12, 8, n)
    e = x.view().dot(y.view())
    r1 = ag.global_sum(e, n, dtype="f32", math=2).cpu().numpy()
    r2 = ag.global_sum(e, n, dtype="f32", math=2).cpu().numpy()
    assert np.array_equal(r1, r2)
    _, exact = oracle_eval(oracle, e, "f32", (), n, op="sum", mode=2)
    assert abs((r1[0] + r1[1]) - (exact[0] + exact[1])) <= 1e-12 * abs(exact[0] + exact[1])
