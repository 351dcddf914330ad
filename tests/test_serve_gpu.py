"""Serving: each request's result is the same alone and in a mix, in batched
and in plain mode, with operands evicted and copied in again under a small
arena; refusals and kept outputs.

Tolerance: bit-exact. A request runs its plan's own arithmetic whatever else
shares its launch, so alone, in a mix and in plain mode must agree bit for
bit; a loose FP64 check against numpy guards against a wrong operand order."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


import aether_gb300 as ag
from aether_gb300 import serve

# The FP64 shapes run in emulated FP64, which carries 48 bits of each input:
# a difference of products of inputs in [-1, 1) is within 2^-44 absolute.
EMU_ATOL = 2.0 ** -44


@pytest.fixture(scope="module")
def shapes():
    return serve.standard_shapes()


@pytest.fixture(scope="module")
def pools():
    return serve.HostPools(f64_bytes=64 << 20, f32_bytes=32 << 20, seed=3)


def _out_buffer(shape, n):
    dt = torch.float64 if shape.out_dtype == "f64" else torch.float32
    return torch.zeros(shape.out_comps * serve.capacity(n), dtype=dt, pin_memory=True)


def _requests(srv, shapes, pools, trace, arrival=False):
    reqs = []
    for s, n, ids, t in trace:
        sh = shapes[s]
        hosts = [pools.window(dt, i, sh.operand_bytes(k, n)) for k, ((dt, _), i) in enumerate(zip(sh.operands, ids))]
        reqs.append(srv.request(s, n, ids, hosts, host_out=_out_buffer(sh, n), arrival_ns=t if arrival else 0))
    return reqs


def _valid(out, n):
    """The n samples of each output plane (the capacity tail is not written)."""
    return out.reshape(-1, serve.capacity(n))[:, :n]


def _alone(shapes, pools, trace, mode="batched", budget=1 << 30):
    outs = []
    with serve.Server(shapes, budget, mode=mode) as srv:
        for r, (_, n, _, _) in zip(_requests(srv, shapes, pools, trace), trace):
            st = srv.wait(srv.submit(r))
            assert st["state"] == "done" and st["launch_items"] == 1
            outs.append(_valid(r.out, n).clone())
    return outs


def _mixed(shapes, pools, trace, mode="batched", budget=1 << 30, **kw):
    with serve.Server(shapes, budget, mode=mode, **kw) as srv:
        reqs = _requests(srv, shapes, pools, trace)
        sts = srv.wait_all(srv.feed(reqs))
        stats = srv.stats()
    assert all(s["state"] == "done" for s in sts)
    return [_valid(r.out, n) for r, (_, n, _, _) in zip(reqs, trace)], sts, stats


def _trace(shapes, n, seed, **kw):
    kw.setdefault("median", 3000)
    kw.setdefault("lo", 64)
    kw.setdefault("hi", 60000)
    return serve.make_trace(shapes, n, None, seed=seed, **kw)


def test_same_alone_in_mix_and_plain(shapes, pools):
    trace = _trace(shapes, 160, seed=21, reuse=0.5)
    alone = _alone(shapes, pools, trace)
    mixed, sts, stats = _mixed(shapes, pools, trace, max_items=64)
    assert max(s["launch_items"] for s in sts) > 1, "the mix never shared a launch"
    for a, m in zip(alone, mixed):
        assert torch.equal(a, m)
    plain, _, pstats = _mixed(shapes, pools, trace, mode="plain")
    assert pstats["launches"] == len(trace)
    for a, p in zip(alone, plain):
        assert torch.equal(a, p)
    # operands through the copy engine instead of the SM gather kernel
    copied, _, _ = _mixed(shapes, pools, trace, max_items=64, upload_engine="copy")
    for a, c in zip(alone, copied):
        assert torch.equal(a, c)
    # one kernel holding every plan instead of one work-list kernel per plan
    one, osts, _ = _mixed(shapes, pools, trace, max_items=64, grouping="mixed")
    assert max(s["launch_items"] for s in osts) > 1
    for a, o in zip(alone, one):
        assert torch.equal(a, o)
    assert stats["resident_hits"] > 0 and stats["completed"] == len(trace)


def test_results_are_right(shapes, pools):
    # loose FP64 checks of two shapes against numpy on the same host bytes
    names = [s.name for s in shapes]
    trace = [(names.index("cross_f64"), 1000, [901, 902], 0), (names.index("expr1_f64"), 777, [903, 904, 905], 0)]
    outs = _alone(shapes, pools, trace)
    a, b = (pools.array("f64", i, 3, 1000) for i in (901, 902))
    ref = np.cross(a.T, b.T).T
    got = outs[0].numpy()
    np.testing.assert_allclose(got, ref, rtol=0, atol=EMU_ATOL)
    a, b, c = (pools.array("f64", i, 3, 777) for i in (903, 904, 905))
    ref = a + b * c + np.sin(a) * np.exp(-(c * c))
    got = outs[1].numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-13)   # emulated sin/exp: ~200 units of 2^-53 of the term scale


def test_small_arena_evicts_and_stays_exact(shapes, pools):
    trace = _trace(shapes, 120, seed=5, reuse=0.7, median=20000, lo=1000, hi=100000)
    alone = _alone(shapes, pools, trace)
    mixed, sts, stats = _mixed(shapes, pools, trace, budget=48 << 20, max_items=32)
    assert stats["evictions"] > 0
    assert stats["arena_peak_bytes"] <= 48 << 20
    for a, m in zip(alone, mixed):
        assert torch.equal(a, m)


def test_refusals_and_kept_outputs(shapes, pools):
    names = [s.name for s in shapes]
    cross = names.index("cross_f64")
    with serve.Server(shapes, 4 << 20, max_inflight=2) as srv:
        big = srv.request(cross, 200000, [1, 2], [pools.window("f64", 1, 3 * 200000 * 8),
                                                  pools.window("f64", 2, 3 * 200000 * 8)])
        with pytest.raises(ag.AetherError, match="budget"):
            srv.submit(big)
        r1 = srv.request(cross, 1000, [7, 8], [pools.window("f64", 7, 3 * 1024 * 8), pools.window("f64", 8, 3 * 1024 * 8)],
                         keep=True)
        t1 = srv.submit(r1)
        st = srv.wait(t1)
        assert st["state"] == "done" and st["output"]
        host = torch.zeros(3 * 1024, dtype=torch.float64, pin_memory=True)
        _abi = ag._abi
        _abi.check(_abi.lib().aether_copy(2, 0, ctypes.c_void_p(host.data_ptr()), 1, 0, ctypes.c_void_p(st["output"]),
                                          host.numel() * 8, None))
        _abi.check(_abi.lib().aether_stream_sync(0, None))
        a, b = pools.array("f64", 7, 3, 1000), pools.array("f64", 8, 3, 1000)
        np.testing.assert_allclose(host.numpy().reshape(3, -1)[:, :1000], np.cross(a.T, b.T).T, rtol=0, atol=EMU_ATOL)
        srv.release(t1)
        assert srv.status(t1)["output"] is None
        # the same id with another size is refused when admitted
        bad = srv.request(cross, 2000, [7, 9], [pools.window("f64", 7, 3 * 2016 * 8), pools.window("f64", 9, 3 * 2016 * 8)])
        with pytest.raises(ag.AetherError, match="resident with"):
            srv.wait(srv.submit(bad))
        # pageable host bytes take the copy engine
        pa, pb = (np.ascontiguousarray(pools.array("f64", i, 3, 1024)) for i in (31, 32))
        pg = srv.request(cross, 1000, [31, 32], [pa.ctypes.data, pb.ctypes.data], keep=True)
        tp = srv.submit(pg)
        stp = srv.wait(tp)
        host2 = torch.zeros(3 * 1024, dtype=torch.float64, pin_memory=True)
        _abi.check(_abi.lib().aether_copy(2, 0, ctypes.c_void_p(host2.data_ptr()), 1, 0, ctypes.c_void_p(stp["output"]),
                                          host2.numel() * 8, None))
        _abi.check(_abi.lib().aether_stream_sync(0, None))
        np.testing.assert_allclose(host2.numpy().reshape(3, -1)[:, :1000], np.cross(pa[:, :1000].T, pb[:, :1000].T).T,
                                   rtol=0, atol=EMU_ATOL)
        srv.release(tp)
        # an id that is resident needs no host bytes
        again = srv.request(cross, 1000, [7, 8], [0, 0])
        assert srv.wait(srv.submit(again))["uploaded_bytes"] == 0


def test_fp64_grade_shapes(pools):
    """Served shapes lowered at FP64 grade (math = 3): each request the same
    alone, in a mix (per-plan work-list kernels of triple-float plans) and in
    plain mode; the large streaming expression within 2 ulp of exact."""
    base = {s.name: s for s in serve.standard_shapes()}
    tf = [serve.ShapeTemplate(name + "_tf", "f64", base[name].out_shape, base[name].operands, base[name].build, math=3)
          for name in ("expr1_f64", "expr2_f64", "cross_f64", "inv3_f64")]
    trace = _trace(tf, 80, seed=8, reuse=0.5)
    alone = _alone(tf, pools, trace)
    mixed, sts, _ = _mixed(tf, pools, trace, max_items=32)
    assert max(s["launch_items"] for s in sts) > 1
    for a, m in zip(alone, mixed):
        assert torch.equal(a, m)
    plain, _, _ = _mixed(tf, pools, trace, mode="plain")
    for a, p in zip(alone, plain):
        assert torch.equal(a, p)
    names = [s.name for s in tf]
    n = 2049
    out = _alone(tf, pools, [(names.index("expr2_f64_tf"), n, [701, 702, 703, 704], 0)])[0].numpy()
    A, B, C, D0 = (np.asarray(pools.array("f64", i, 3, n), dtype=np.longdouble) for i in (701, 702, 703, 704))
    t1 = np.sqrt(A * A + B * B) * np.log1p(np.abs(C))
    t2 = 1 / np.sqrt(1 + D0 * D0)
    exact = t1 + t2
    mag = np.maximum(np.abs(exact), np.maximum(np.abs(t1), np.abs(t2))).astype(np.float64)
    err = np.abs(np.asarray(out, dtype=np.longdouble) - exact) / np.spacing(mag)
    assert float(err.max()) <= 2.0
