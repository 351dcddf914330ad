"""Sharding the sample axis across ranks (one process per GPU).

The fused-expression path needs no exchange: samples are independent, so
rank r evaluates block r of every array's sample mode (partition_view of
residency/Partition.h:104-168) or, for weak scaling, its own replica. The
only cross-rank step is a global compensated sum, one (hi, comp) pair per
rank, combined here in rank order with the same pair combination the
device's warp tree uses (accum/atomic.h:141-160), so every rank gets the
same bits whatever the world size's reduction tree would have done.
These helpers take an initialised torch.distributed group (nccl on GPUs,
gloo on CPUs) or None for a single process.
"""

import math

from . import padded_block_samples


def shard_samples(n, rank, world, pad_to=32):
    """(first sample, count) of rank's block of n samples: block pitch
    ceil(n / world) rounded up to pad_to, the last block short."""
    pitch = padded_block_samples(n, world, pad_to)
    off = rank * pitch
    return min(off, n), max(0, min(pitch, n - off))


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def pair_combine(ah, ac, bh, bc):
    """(ah, ac) + (bh, bc) as a compensated pair (the host twin of the
    device's pair_combine)."""
    s, e = _two_sum(ah, bh)
    return s, ((ac + bc) + e) if math.isfinite(s) else 0.0


def max_over_ranks(value, group=None):
    """The largest of each rank's value (timings: the slowest rank sets the
    job's time)."""
    import torch
    import torch.distributed as dist
    if group is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def global_sum(hi, comp, group=None):
    """Combine each rank's (hi, comp) pair into the job's sum, identically on
    every rank: all pairs are gathered and folded in rank order."""
    import torch
    import torch.distributed as dist
    if group is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(hi), float(comp)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    mine = torch.tensor([float(hi), float(comp)], dtype=torch.float64, device=dev)
    parts = [torch.empty_like(mine) for _ in range(dist.get_world_size())]
    dist.all_gather(parts, mine)
    h, c = 0.0, 0.0
    for p in parts:
        ph, pc = p.tolist()
        h, c = pair_combine(h, c, ph, pc)
    return h, c
