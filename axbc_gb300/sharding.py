"""Pivot sharding across GPUs (one process per GPU).

Pivots are independent, so every rank keeps a replica of the graph, computes
bc over its own share of the pivots, and the ranks' bc vectors are summed once
at the end -- the reference's cluster replicas (src/axbc2d.c:2438, 2836
`ui += cntask`, and the final MPI_Reduce of bc, 3159-3167).  Timing across
ranks takes the maximum.  Works with any torch.distributed backend (NCCL on
GPUs, gloo on CPU).
"""
from __future__ import annotations

import os


def env():
    """(rank, world, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(seq, rank: int, world: int):
    """The rank's pivots: every world-th one from position rank (ui += cntask)."""
    return seq[rank::world]


def rank_seed(seed: int, rank: int) -> int:
    """Seed of a rank's own pivot stream in sampled runs."""
    return seed + rank


def sum_bc(bc, group=None):
    """In-place sum of the ranks' bc tensors (float32)."""
    import torch.distributed as dist
    if dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(bc, op=dist.ReduceOp.SUM, group=group)
    return bc


def max_time(seconds: float, device=None) -> float:
    """Largest elapsed time over the ranks."""
    import torch
    import torch.distributed as dist
    if not (dist.is_initialized() and dist.get_world_size() > 1):
        return seconds
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def total(x: float, device=None) -> float:
    """Sum of a per-rank count over the ranks."""
    import torch
    import torch.distributed as dist
    if not (dist.is_initialized() and dist.get_world_size() > 1):
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t)
    return float(t.item())
