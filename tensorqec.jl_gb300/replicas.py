"""Replicas across GPUs: the decoder shards by syndrome, with no data exchange.

Each rank decodes its own syndromes with its own copy of the program; the
only cross-rank operation is a reduction of per-step times (the slowest rank
sets the step) and of counters (logical errors, fallbacks).  Sample streams
are disjoint by construction: the GPU sampler is counter-based, so rank r of
a job that draws n samples per rank takes sample indices [r*n, (r+1)*n); host
sampling uses a seed per rank.
"""
from __future__ import annotations


def rank_seed(base_seed: int, rank: int) -> int:
    """Seed of rank `rank`'s host sample stream."""
    return int(base_seed) + int(rank)


def sample_offset(rank: int, n_per_rank: int) -> int:
    """First sample index of rank `rank` in the counter-based GPU sampler."""
    return int(rank) * int(n_per_rank)


def reduce_max(values, dist=None, device=None):
    """Element-wise maximum over ranks (the slowest rank's step times)."""
    vals = [float(v) for v in values]
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return vals
    import torch

    t = torch.tensor(vals, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def reduce_sum(values, dist=None, device=None):
    """Element-wise sum over ranks (logical errors, fallback rows)."""
    vals = [int(v) for v in values]
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return vals
    import torch

    t = torch.tensor(vals, dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return [int(x) for x in t.tolist()]


def job_rate(world: int, batch: int, step_ms: float) -> float:
    """Whole-job syndromes/s: every rank decodes `batch` syndromes per step."""
    return world * batch / (step_ms / 1e3)
