"""Serving host logic without a GPU: the mixed-request trace (arrivals, size
distribution, operand reuse) and the serving entry points' presence."""

import types

import numpy as np

from aether_gb300 import serve


def _fake_shapes():
    return [types.SimpleNamespace(operands=[("f64", (3,))] * k) for k in (1, 2, 3, 4, 2, 2, 2, 1)]


def test_trace_is_seeded_and_poisson():
    sh = _fake_shapes()
    t1 = serve.make_trace(sh, 4000, 10000.0, seed=4)
    t2 = serve.make_trace(sh, 4000, 10000.0, seed=4)
    assert t1 == t2
    arr = np.array([t for *_, t in t1], dtype=np.float64)
    assert np.all(np.diff(arr) >= 0)
    gaps = np.diff(arr) / 1e9
    assert abs(gaps.mean() - 1e-4) < 1e-5          # rate 10k/s
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.1  # exponential gaps


def test_trace_sizes_and_reuse():
    sh = _fake_shapes()
    tr = serve.make_trace(sh, 6000, None, seed=9, reuse=0.7)
    ns = np.array([n for _, n, _, _ in tr])
    assert ns.min() >= 1024 and ns.max() <= 4194304
    seen, reused = set(), 0
    for s, n, ids, t in tr:
        assert t == 0
        assert len(ids) == len(sh[s].operands)
        key = tuple(ids)
        reused += key in seen
        seen.add(key)
    # the first request of each shape cannot reuse; the rest reuse with p = 0.7
    assert abs(reused / len(tr) - 0.7) < 0.03
    assert 40000 < np.median(ns) < 110000


def test_capacity_rule():
    assert serve.capacity(1) == 32 and serve.capacity(32) == 32 and serve.capacity(33) == 64
