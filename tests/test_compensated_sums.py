"""Compensated sums against exactly known answers, the construction of the
reference's own fixtures (tests/test_CompensatedSum_common.h:33-56): pairs
+x, -x of full-precision values in [1, 3) that cancel exactly, plus residual
terms on a 2^-10 grid whose sum is known, shuffled. A plain running sum loses
the residuals; the Neumaier walk and the fixed 32-slot tree keep them within
one ulp (:97-112). The pair combination is bitwise symmetric and keeps a
residual far below its partner (:114-140).

CPU: the oracle's restatement of the primitives (oracle/aether_oracle.cpp).
GPU: the engine's sum plans (per-thread Neumaier, the pair tree, the FP64
final stage) over the same terms in device arrays."""

import ctypes
import math

import numpy as np
import pytest


def make_fixture(seed, dtype=np.float64, pairs=64, residuals=64):
    rng = np.random.default_rng(seed)
    x = rng.uniform(1.0, 3.0, pairs).astype(dtype)
    g = rng.integers(1, 5, residuals)
    terms = np.concatenate([x, -x, (g * 0.0009765625).astype(dtype)])
    rng.shuffle(terms)
    return terms, float(g.sum()) * 0.0009765625


def ulp_err(got, exact, dtype=np.float64):
    e = dtype(exact)
    return abs(float(got) - exact) / float(np.spacing(e))


def walk(oracle, terms):
    h, c = ctypes.c_double(0.0), ctypes.c_double(0.0)
    for t in terms:
        oracle.lib().orc_neumaier_add_f64(ctypes.byref(h), ctypes.byref(c), ctypes.c_double(float(t)))
    return h.value + c.value


def tree(oracle, terms):
    h, c = np.zeros(32), np.zeros(32)
    hp, cp = ctypes.c_double(), ctypes.c_double()
    for i, t in enumerate(terms):
        hp.value, cp.value = h[i % 32], c[i % 32]
        oracle.lib().orc_neumaier_add_f64(ctypes.byref(hp), ctypes.byref(cp), ctypes.c_double(float(t)))
        h[i % 32], c[i % 32] = hp.value, cp.value
    oh, oc = ctypes.c_double(), ctypes.c_double()
    oracle.lib().orc_reduce32_f64(h.ctypes.data, c.ctypes.data, ctypes.byref(oh), ctypes.byref(oc))
    return oh.value + oc.value


@pytest.mark.parametrize("seed", range(1, 9))
def test_walk_and_tree_within_one_ulp(oracle, seed):
    terms, exact = make_fixture(seed)
    assert math.fsum(terms) == exact
    assert ulp_err(walk(oracle, terms), exact) <= 1.0
    assert ulp_err(tree(oracle, terms), exact) <= 1.0


def test_plain_sum_fails_the_fixture():
    failures = 0
    for seed in range(1, 9):
        terms, exact = make_fixture(seed)
        s = 0.0
        for t in terms:
            s += float(t)
        failures += ulp_err(s, exact) > 1.0
    assert failures >= 6


def test_pair_combine_symmetric_and_keeps_the_residual(oracle):
    rng = np.random.default_rng(7)
    f = oracle.lib().orc_pair_combine_f64
    xh, xc, yh, yc = (ctypes.c_double() for _ in range(4))
    for i in range(20000):
        ah = rng.uniform(-1, 1) * 2.0 ** (i % 20 - 10)
        bh = rng.uniform(-1, 1) * 2.0 ** ((i // 7) % 20 - 10)
        ac, bc = rng.uniform(-1, 1) * 1e-6, rng.uniform(-1, 1) * 1e-6
        f(ctypes.c_double(ah), ctypes.c_double(ac), ctypes.c_double(bh), ctypes.c_double(bc), ctypes.byref(xh),
          ctypes.byref(xc))
        f(ctypes.c_double(bh), ctypes.c_double(bc), ctypes.c_double(ah), ctypes.c_double(ac), ctypes.byref(yh),
          ctypes.byref(yc))
        assert xh.value == yh.value and xc.value == yc.value, i
    big, tiny = 2.0 ** 56, 0.0009765625
    f(ctypes.c_double(big), ctypes.c_double(0.0), ctypes.c_double(tiny), ctypes.c_double(0.0), ctypes.byref(xh),
      ctypes.byref(xc))
    assert xh.value == big and xc.value == tiny


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(1, 9))
@pytest.mark.parametrize("reps", [1, 4096])
def test_engine_sum_plans_on_the_fixture(seed, reps):
    """The fixture tiled `reps` times across one array (so every thread and
    the tree see cancelling pairs), summed by a sum plan: within one ulp of
    the exact total, the same bits on a second launch."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import aether_gb300 as ag
    terms, exact = make_fixture(seed)
    rng = np.random.default_rng(seed + 100)
    tiled = np.tile(terms, reps)
    rng.shuffle(tiled)
    x = ag.Array("f64", (1,), tiled.size)
    x.upload(tiled[None, :])
    r1 = ag.global_sum(x.view().sum(), tiled.size).cpu().numpy()
    r2 = ag.global_sum(x.view().sum(), tiled.size).cpu().numpy()
    assert np.array_equal(r1, r2)
    assert ulp_err(r1[0] + r1[1], exact * reps) <= 1.0
