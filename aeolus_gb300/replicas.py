"""Replica sharding across GPUs (one process per GPU, no data-path
collective): every rank advances its own members; only the timing is
reduced.  The reference runs one state per process, so this is the
multi-GPU form of its run loop (run/engine.py:406-431) for independent
members."""
from __future__ import annotations


def member_seed_base(rank: int, members: int) -> int:
    """Seed base of rank `rank`: workloads.member_states gives member b the
    seed base + 1000 b, so rank r owns seeds 1000 (r * members + b) and no
    two ranks share a member."""
    return 1000 * members * int(rank)


def max_over_ranks(value: float, device=None) -> float:
    """Max of a per-rank timing over the process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
