"""Multi-GPU host logic for the batched path: one process per GPU.

The batched Newton workload is independent circuit instances, so ranks do
not exchange data: every rank solves its own seeded batch of the same size
(weak scaling), and the only collective is the reduction of the step time
to its maximum over ranks for reporting.
"""
from __future__ import annotations


def shard_seed(rank: int, base: int = 3) -> int:
    """Seed of rank ``rank``'s batch; rank 0 keeps the single-GPU workload."""
    return base + 7919 * rank


def max_over_ranks(value: float, device=None) -> float:
    """Max of ``value`` over the default process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    """Sum of ``value`` over the default process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
