"""Work split across GPUs for independent molecules.

The RHF path shards by molecule (each SCF is independent), so N GPUs run N
disjoint slices of a molecule list with no data exchange; only timing uses
a collective (max over ranks).  ``shard`` gives rank r the molecules
``order[r::world]`` of a longest-first ordering, which balances uneven
molecule sizes.
"""
from __future__ import annotations

from typing import Sequence


def shard(costs: Sequence[float], world: int, rank: int):
    """Indices of the molecules rank ``rank`` of ``world`` runs (cost-balanced)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad world/rank")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    return sorted(order[rank::world])


def max_over_ranks(value: float) -> float:
    """Max of ``value`` over the default torch.distributed group (or itself)."""
    try:
        import torch
        import torch.distributed as dist
    except ImportError:
        return value
    if not (dist.is_available() and dist.is_initialized()):
        return value
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
