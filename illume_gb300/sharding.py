"""Replica sharding across GPUs (one process per GPU).

Every (pixel, sample) path is independent and its random numbers are keyed by (pixel,
sample, bounce), so a render shards by sample ranges with no exchange on the data path:
each rank renders a disjoint range of samples of the same frame, and the only exchange
is one sum of the per-pixel accumulators at the end (or none, for throughput runs).
"""
from __future__ import annotations


def shard_samples(spp: int, rank: int, world: int) -> tuple[int, int]:
    """(first sample, sample count) of `rank` when `spp` samples are split over `world`."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    base, extra = divmod(spp, world)
    begin = rank * base + min(rank, extra)
    return begin, base + (1 if rank < extra else 0)


def replica_sample_base(rank: int, stride: int = 1_000_000) -> int:
    """First sample of a weak-scaling replica: ranks never share (pixel, sample) streams."""
    return rank * stride


def reduce_sums(sum_rgb, sumsq_rgb, group=None):
    """Sum per-pixel accumulators (numpy float64) over ranks with torch.distributed."""
    import numpy as np
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(np.stack([sum_rgb, sumsq_rgb]))).double()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out = t.numpy()
    return out[0], out[1]


def max_over_ranks(value: float, group=None) -> float:
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t[0])
