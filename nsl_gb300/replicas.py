"""Replica bookkeeping for runs with one process per GPU.

The fermion-matrix work shards into independent units (configurations, chains, right-hand-side blocks) that share
nothing but the read-only exp(delta K), so ranks exchange no data: each rank processes its own units, and only the
timing is reduced. The slowest rank defines the job time; the job rate counts the units of all ranks.
"""
from __future__ import annotations


def shard(n_units: int, rank: int, world: int) -> range:
    """The contiguous block of units rank `rank` of `world` owns (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    base, extra = divmod(int(n_units), int(world))
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(seconds: float, dist=None, device=None) -> float:
    """The largest of the ranks' times (the job time); the local time without a process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(seconds)
    import torch

    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, seconds: float, dist=None, device=None) -> float:
    """Units of all ranks per second of the slowest rank (weak scaling: every rank processes units_per_rank)."""
    world = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    return world * float(units_per_rank) / max_over_ranks(seconds, dist, device)
