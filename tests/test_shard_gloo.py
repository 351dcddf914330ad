"""The multi-rank host logic on CPU with two gloo ranks: shards cover the
sample axis exactly once, timings reduce to the slowest rank, and a global
compensated sum combines per-rank pairs to the same bits on every rank and
to the exactly rounded total."""

import math
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from aether_gb300 import shard  # noqa: E402


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n = 100003
        off, cnt = shard.shard_samples(n, rank, world)
        slowest = shard.max_over_ranks(10.0 + rank, group=dist.group.WORLD)
        rng = np.random.default_rng(7)
        data = rng.standard_normal(n) * 10.0 ** rng.uniform(-8, 8, n)
        h, c = 0.0, 0.0
        for x in data[off:off + cnt]:          # this rank's compensated partial
            s, e = shard._two_sum(h, x)
            h, c = s, c + e
        gh, gc = shard.global_sum(h, c, group=dist.group.WORLD)
        out[rank] = (off, cnt, slowest, gh, gc, math.fsum(data))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = [out[r] for r in range(world)]
    spans = sorted((o, c) for o, c, *_ in res)
    assert spans[0][0] == 0 and spans[0][0] + spans[0][1] == spans[1][0]
    assert spans[1][0] + spans[1][1] == 100003
    assert all(r[2] == 11.0 for r in res)
    assert res[0][3:5] == res[1][3:5]              # the same bits on every rank
    total = res[0][3] + res[0][4]
    assert abs(total - res[0][5]) <= 4 * abs(np.spacing(res[0][5]))


def test_single_process_fallbacks():
    assert shard.shard_samples(100, 0, 1) == (0, 100)
    assert shard.shard_samples(100, 3, 4) == (96, 4)
    assert shard.max_over_ranks(3.5) == 3.5
    assert shard.global_sum(1.0, 1e-20) == (1.0, 1e-20)
