"""Independence of the Philox streams (tests/test_RandomIndependence.cpp).

Each (seed, global, counter) owns one Philox block and every draw reads only
that block's words, so neighbouring counters are independent.

CPU (the oracle, the reference's primitives restated): the lag-k fourth
moment E[z^2 z'^2] = 1 of standard normals k counters apart, double and float
(:29-58); the words of 256 consecutive blocks are all distinct (:60-76); the
64-bit and uniform primitives read their own block's words and neighbouring
counters share none (:78-95); uniforms stay inside the open interval at the
boundary words, with finite logarithms of the draw and its complement
(:97-116).

GPU: the same moment over the engine's own normal fills, for samples `lag`
apart (consecutive globals) and for the components of one sample
(consecutive counters), in the native and the emulated lowerings and in
float storage."""

import math

import numpy as np
import pytest

LAGS = [1, 2, 3, 4, 5, 6, 7, 8, 16, 64]
SEEDS = [0, 0xC0FFEE, 0xFFFFFFFFFFFFFFFF]


@pytest.mark.parametrize("f32,salt", [(False, 0x1234567), (True, 0x7654321)])
def test_lag_fourth_moment(oracle, f32, salt):
    for lag in LAGS:
        mean, se = oracle.lag_fourth_moment(salt, lag, 1000000, f32)
        assert abs(mean - 1.0) < 5.0 * se, (lag, mean, se)


def test_blocks_are_word_disjoint_across_counters(oracle):
    for seed in SEEDS:
        for g in (0, 3, 0xFFFFFFFF):
            words = np.concatenate([oracle.philox_block(seed, g, c) for c in range(256)])
            assert np.unique(words).size == words.size, (seed, g)


def test_primitives_read_only_their_own_block(oracle):
    L = oracle.lib()
    for seed in SEEDS:
        for c in range(512):
            b = oracle.philox_block(seed, 7, c)
            assert L.orc_random_bits64(seed, 7, c) == (int(b[1]) << 32) | int(b[0])
            assert L.orc_uniform01_f64(seed, 7, c) == L.orc_u01_from_word_f64(int(b[0]))
            assert L.orc_uniform01_f32(seed, 7, c) == L.orc_u01_from_word_f32(int(b[0]))
            assert L.orc_random_bits64(seed, 7, c) >> 32 != L.orc_random_bits64(seed, 7, c + 1) & 0xFFFFFFFF


def test_uniforms_open_interval_at_boundary_words(oracle):
    L = oracle.lib()
    words = [0, 1, 0x1FF, 0x200, 0x7FFFFFFF, 0x80000000, 0xFFFFFE00, 0xFFFFFFFE, 0xFFFFFFFF]
    for w in words:
        d, f = L.orc_u01_from_word_f64(w), L.orc_u01_from_word_f32(w)
        assert 0.0 < d < 1.0 and 0.0 < f < 1.0, w
    assert L.orc_u01_from_word_f32(0) <= L.orc_u01_from_word_f32(0xFFFFFFFF)
    assert L.orc_u01_from_word_f64(0) <= L.orc_u01_from_word_f64(0xFFFFFFFF)
    for w in (0, 0xFFFFFFFF):
        d = L.orc_u01_from_word_f64(w)
        assert math.isfinite(math.log(d)) and math.isfinite(math.log(1.0 - d))
        f = np.float32(L.orc_u01_from_word_f32(w))
        assert np.isfinite(np.log(np.float32(1.0) - f))
    # the Box-Muller uniform (53 bits from two words) at its extremes
    for x, y in ((0, 0), (0xFFFFFFFF, 0xFFFFFFFF), (0, 0xFFFFFFFF), (0xFFFFFFFF, 0)):
        u = L.orc_u01_hq(x, y)
        assert 0.0 < u < 1.0 and math.isfinite(math.log(u)), (x, y)


def _moment(torch, z, y):
    q = (z * z * y * y).double()
    n = q.numel()
    mean = float(q.mean())
    se = math.sqrt(max(float((q * q).mean()) - mean * mean, 0.0) / n)
    return mean, se


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,math_", [("f64", 0), ("f64", 1), ("f32", 0)])
def test_engine_fills_lag_fourth_moment(dtype, math_):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import aether_gb300 as ag
    n = 1 << 22
    x = ag.Array(dtype, (2,), n)
    ag.assign(x, ag.Generator(0x5EED).substream(3).normal(2, 0.0, 1.0), math=math_)
    z0, z1 = x.data[0, :n], x.data[1, :n]
    assert abs(float(z0.double().mean())) < 5.0 / math.sqrt(n)
    for lag in LAGS:
        mean, se = _moment(torch, z0[:-lag], z0[lag:])   # samples lag apart: consecutive globals
        assert abs(mean - 1.0) < 5.0 * se, (lag, mean, se)
    mean, se = _moment(torch, z0, z1)                    # components: consecutive counters
    assert abs(mean - 1.0) < 5.0 * se, (mean, se)
