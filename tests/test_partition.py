"""Sample-mode partitions (residency/Partition.h:52-168): the block pitch and
the closed-form block views on the reference's cases, and, on the device,
an expression evaluated block by block equals the whole-array launch bit for
bit (each sample's arithmetic does not depend on where the launch starts)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import aether_gb300 as ag


def test_padded_block_samples_reference_cases():
    assert ag.padded_block_samples(100, 4, 32) == 32
    assert ag.padded_block_samples(100, 3, 32) == 64
    assert ag.padded_block_samples(96, 3, 32) == 32
    assert ag.padded_block_samples(10, 4) == 32
    assert ag.padded_block_samples(10, 4, 4) == 4
    assert ag.padded_block_samples(10, 4, 1) == 3
    with pytest.raises(ag.AetherError, match="parts must be > 0"):
        ag.padded_block_samples(100, 0, 32)
    with pytest.raises(ag.AetherError, match="pad_to must be > 0"):
        ag.padded_block_samples(100, 4, 0)


def test_partition_view_closed_form():
    full = ag.Array("f64", (3,), 100, device="cpu")
    full.data[:, :100] = torch.arange(100, dtype=torch.float64)[None, :] + 1000.0 * torch.arange(3)[:, None]
    off, real = [0, 32, 64, 96], [32, 32, 32, 4]
    for r in range(4):
        b = ag.partition_view(full, 4, r)
        assert b.n == real[r]
        assert b.capacity == full.capacity
        assert b.data.data_ptr() == full.data.data_ptr() + off[r] * 8
        assert np.array_equal(b.host(), full.host()[:, off[r]:off[r] + real[r]])
    with pytest.raises(ag.AetherError, match="block index 4 >= spec.parts=4"):
        ag.partition_view(full, 4, 4)


@pytest.mark.gpu
def test_blockwise_launches_equal_whole():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n = 100003
    g = ag.Generator(42)
    arrs = [ag.Array("f64", (3,), n) for _ in range(3)]
    for k, x in enumerate(arrs):
        ag.assign(x, g.substream(k).uniform(3, -1.0, 1.0))
    whole = ag.Array("f64", (3,), n)

    def expr(a, b, c):
        a, b, c = a.view(), b.view(), c.view()
        return a + b * c + ag.cwiseSin(a) * ag.cwiseExp((c * c) * (-1.0))

    ag.assign(whole, expr(*arrs), math=1)
    parts = ag.Array("f64", (3,), n)
    for r in range(7):
        blocks = [ag.partition_view(x, 7, r) for x in arrs + [parts]]
        if blocks[0].n:
            ag.assign(blocks[3], expr(*blocks[:3]), math=1)
    torch.cuda.synchronize()
    assert np.array_equal(parts.host(), whole.host())
    # random leaves keep their global sample index through sample_offset
    z = ag.Array("f64", (1,), n)
    zb = ag.Array("f64", (1,), n)
    leaf = g.substream(9).normal(1, 0.0, 1.0)
    ag.assign(z, leaf)
    pitch = ag.padded_block_samples(n, 5)
    for r in range(5):
        b = ag.partition_view(zb, 5, r)
        if b.n:
            ag.prepare(b, leaf, sample_offset=r * pitch)()
    torch.cuda.synchronize()
    assert np.array_equal(zb.host(), z.host())


def test_dlpack_round_trip_zero_copy():
    a = ag.Array("f64", (3,), 100, device="cpu")
    a.data[:, :100] = torch.arange(300, dtype=torch.float64).reshape(3, 100)
    t = torch.from_dlpack(a)
    assert t.shape == (3, 100) and t.stride() == (a.capacity, 1) and t.data_ptr() == a.data.data_ptr()
    b = ag.Array.from_dlpack(torch.zeros(3, 128, dtype=torch.float64), shape=(3,), n=100)
    assert b.capacity == 128 and b.n == 100
