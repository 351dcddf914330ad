"""Batches: uneven arrays of three expression kinds (cross product,
quaternion rotation, guarded 3x3 inverse) in one persistent launch, and that
launch replayed from a CUDA graph. Each item's result must equal the plain
per-item launch of the same plan bit for bit, and the oracle's."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


import aether_gb300 as ag


def make_workload(n_items, median, sigma, lo, hi, seed, math=0):
    rng = np.random.default_rng(seed)
    sizes = np.clip(np.round(rng.lognormal(np.log(median), sigma, n_items)), lo, hi).astype(int)
    g = ag.Generator(seed)
    items = []
    for i, n in enumerate(sizes):
        kind = i % 3
        gi = g.substream(i)
        if kind == 0:
            a, b = ag.Array("f64", (3,), n), ag.Array("f64", (3,), n)
            ag.assign(a, gi.substream(0).uniform(3, -1.0, 1.0))
            ag.assign(b, gi.substream(1).uniform(3, -1.0, 1.0))
            out = ag.Array("f64", (3,), n)
            expr = a.view().cross(b.view())
            ins = (a, b)
        elif kind == 1:
            q, v = ag.Array("f64", (4,), n), ag.Array("f64", (3,), n)
            ag.assign(q, gi.substream(0).uniform(4, -1.0, 1.0))
            ag.assign(v, gi.substream(1).uniform(3, -1.0, 1.0))
            out = ag.Array("f64", (3,), n)
            expr = q.view().quatRotate(v.view())
            ins = (q, v)
        else:
            m = ag.Array("f64", (3, 3), n)
            ag.assign(m, gi.substream(0).uniform(9, -1.0, 1.0).reshape((3, 3)))
            out = ag.Array("f64", (3, 3), n)
            M = m.view()
            expr = ag.select(ag.cwiseAbs(M.det()) > 1e-300, M.inverse(), ag.constant(0.0, (3, 3)))
            ins = (m,)
        items.append((out, expr, ins))
    return items


@pytest.mark.parametrize("math", [0, 1, 3])
def test_batch_equals_per_item_launches_and_graph_replay(math):
    work = make_workload(300, 600, 1.5, 1, 40000, seed=3, math=math)
    launches = [ag.prepare(out, e, math=math) for out, e, _ in work]
    # per-item launches into reference buffers
    refs = []
    for (out, e, _), L in zip(work, launches):
        L()
    torch.cuda.synchronize()
    refs = [out.data[:, : out.n].clone() for out, _, _ in work]
    for out, _, _ in work:
        out.data.zero_()
    batch = ag.Batch(launches)
    info = batch.info()
    assert info.n_plans == 3 and info.n_items == 300
    batch.launch()
    torch.cuda.synchronize()
    for (out, _, _), r in zip(work, refs):
        assert torch.equal(out.data[:, : out.n], r)
    # graph capture and replay
    for out, _, _ in work:
        out.data.zero_()
    s = torch.cuda.Stream()
    batch.capture(s.cuda_stream)
    batch.replay(s.cuda_stream)
    s.synchronize()
    for (out, _, _), r in zip(work, refs):
        assert torch.equal(out.data[:, : out.n], r)
    # new input contents, same tiling: the graph reads them
    out0, _, ins0 = work[0]
    ins0[0].data.mul_(2.0)
    batch.replay(s.cuda_stream)
    s.synchronize()
    assert torch.allclose(out0.data[:, : out0.n], 2.0 * refs[0])


def test_batch_matches_oracle(oracle):
    work = make_workload(60, 300, 1.0, 1, 5000, seed=9)
    launches = [ag.prepare(out, e, contract=0) for out, e, _ in work]
    batch = ag.Batch(launches)
    batch.launch()
    torch.cuda.synchronize()
    for out, e, ins in work:
        ctx = ag.IrContext()
        ir = ag.expr.plan_text("f64", out.shape, "set", e, ctx)
        ops = [np.ascontiguousarray(owner.data.cpu().numpy()) for (_, _, _, _, owner) in ctx.operands]
        ref, _ = oracle.eval_ir(ir, out.n, ops, scalars=ctx.scalars, dst_comps=out.comps)
        assert np.array_equal(out.host(), ref[:, : out.n])


def test_batch_rejects_sum_plans_and_misaligned_items():
    x = ag.Array("f64", (3,), 100)
    s = ag.Array("f64", (1,), 100)
    red = torch.zeros(2, dtype=torch.float64, device="cuda")
    Ls = ag.prepare(s, x.view().dot(x.view()), op="setsum", reduce_out=red)
    with pytest.raises(ag.AetherError, match="sum plans"):
        ag.Batch([Ls])
    base = torch.zeros((3, 200), dtype=torch.float64, device="cuda")
    mis = ag.expr.Operand(base.data_ptr() + 8, 200, "f64", (3,))
    d = ag.Array("f64", (3,), 100)
    with pytest.raises(ag.AetherError, match="aligned"):
        ag.Batch([ag.prepare(d, mis * 2.0)])
