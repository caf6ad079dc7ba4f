"""Sample sharding across processes (one GPU each): every rank renders the same
scene with its own sample keys, and the only exchange is one sum of the float4
accumulators (rgb sums and sample counts) when an image is wanted. The path
has no other cross-rank dependency, so the benchmark's multi-GPU form is
weak-scaled shards with no collective on the data path."""
from __future__ import annotations

from dataclasses import replace

from .renderer import KernelSettings

SEED_STRIDE = 7919  # prime offset between the ranks' seeds


def shard_settings(settings: KernelSettings, rank: int) -> KernelSettings:
    """The settings of one shard: the counter RNG is keyed by (pixel, sample, bounce, seed),
    so a distinct seed per rank gives disjoint sample streams."""
    return replace(settings, seed=(settings.seed + SEED_STRIDE * rank) & 0xFFFFFFFF)


def reduce_accumulators(acc, group=None):
    """Sums the ranks' accumulators (a float32 tensor (..., 4): rgb sums, sample count) in
    place with one all-reduce and returns it; colors = acc[..., :3] / acc[..., 3:]."""
    import torch.distributed as dist

    dist.all_reduce(acc, op=dist.ReduceOp.SUM, group=group)
    return acc


def max_over_ranks(value: float, device="cpu", group=None) -> float:
    """The largest of the ranks' values (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
