"""The Python front end's remaining Expression members (expr/Expression.h:
rSquaredNorm, cubedNorm, rCubedNorm :182-184, matDot :205-207,
quatReciprocal :220-222, asBack3DVector :228), built from the node set.

CPU: the IR each writes, evaluated by the oracle, against numpy's formula.
GPU: the engine's kernel against the oracle on the same inputs, bit for bit
with contraction off."""

import numpy as np
import pytest

import aether_gb300 as ag
from aether_gb300.expr import IrContext, Operand, plan_text

N = 257


def _inputs():
    rng = np.random.default_rng(1)
    return rng.uniform(-1, 1, (4, N)), rng.uniform(-1, 1, (9, N)), rng.uniform(-1, 1, (9, N))


def _cases(q, m, mm):
    return {
        "quatReciprocal": (q.quatReciprocal(), (4,), ["Q"]),
        "asBack3DVector": (q.asBack3DVector(), (3,), ["Q"]),
        "rSquaredNorm": (q.rSquaredNorm(), (), ["Q"]),
        "cubedNorm": (q.cubedNorm(), (), ["Q"]),
        "rCubedNorm": (q.rCubedNorm(), (), ["Q"]),
        "matDot": (m.matDot(mm), (), ["M", "N"]),
    }


def _numpy(name, Q, M, N_):
    s = (Q * Q).sum(0)
    return {
        "quatReciprocal": np.stack([Q[0], -Q[1], -Q[2], -Q[3]]) / s,
        "asBack3DVector": Q[1:4],
        "rSquaredNorm": (1 / s)[None],
        "cubedNorm": (s * np.sqrt(s))[None],
        "rCubedNorm": (1 / (s * np.sqrt(s)))[None],
        "matDot": (M * N_).sum(0)[None],
    }[name]


NAMES = ["quatReciprocal", "asBack3DVector", "rSquaredNorm", "cubedNorm", "rCubedNorm", "matDot"]


@pytest.mark.parametrize("name", NAMES)
def test_members_through_the_oracle(oracle, name):
    Q, M, N_ = _inputs()
    q = Operand(0x1000, N, "f64", (4,))
    m, mm = Operand(0x2000, N, "f64", (3, 3)), Operand(0x3000, N, "f64", (3, 3))
    e, shape, ops = _cases(q, m, mm)[name]
    ctx = IrContext()
    ir = plan_text("f64", shape, "set", e, ctx)
    arrays = {"Q": Q, "M": M, "N": N_}
    comps = int(np.prod(shape)) if shape else 1
    d, _ = oracle.eval_ir(ir, N, [np.ascontiguousarray(arrays[k]) for k in ops], scalars=ctx.scalars, dst_comps=comps)
    ref = _numpy(name, Q, M, N_)
    assert np.allclose(d, ref, rtol=4e-16, atol=0), name


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_members_on_device(oracle, name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    Q, M, N_ = _inputs()
    arrs = {}
    for k, (h, shape) in {"Q": (Q, (4,)), "M": (M, (3, 3)), "N": (N_, (3, 3))}.items():
        a = ag.Array("f64", shape, N)
        a.upload(h)
        arrs[k] = a
    e, shape, ops = _cases(arrs["Q"].view(), arrs["M"].view(), arrs["N"].view())[name]
    d = ag.Array("f64", shape if shape else (1,), N)
    ag.assign(d, e, contract=0)
    ctx = IrContext()
    ir = plan_text("f64", shape, "set", e, ctx)
    comps = int(np.prod(shape)) if shape else 1
    host = {"Q": Q, "M": M, "N": N_}
    ref, _ = oracle.eval_ir(ir, N, [np.ascontiguousarray(host[k]) for k in ops], scalars=ctx.scalars, dst_comps=comps)
    assert np.array_equal(d.host(), ref[:, :N]), name
