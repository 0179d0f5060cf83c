"""Replica bookkeeping for runs on several GPUs of one node.

Frames and sprites are independent units with no exchange step, so several
GPUs run as replicas: each rank takes its own share of the units (or its own
copy of a fixed per-rank workload), the ranks meet at a barrier around the
timed region, and the job's time is the slowest rank's. Nothing on the data
path crosses ranks; the only collectives are these host-side reductions.
"""
from __future__ import annotations


def shard(n_units: int, rank: int, world: int) -> range:
    """Units [start, end) of `rank` when `n_units` are split over `world`
    ranks as evenly as possible (the first n_units % world ranks take one
    more)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over all ranks (the value itself without an
    initialised process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_throughput(units_this_rank: float, seconds_this_rank: float, device=None) -> float:
    """Whole-job units per second: every rank's units over the slowest
    rank's time."""
    total = sum_over_ranks(units_this_rank, device)
    slowest = max_over_ranks(seconds_this_rank, device)
    return total / slowest if slowest > 0 else 0.0
