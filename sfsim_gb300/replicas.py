"""Multi-GPU use of the LUT build: independent replicas.

Every scattering order needs the whole previous-order table, and one build
takes tens of milliseconds, so a single build is not split across GPUs.  What
does spread over GPUs is independent work: whole builds (replicas) and the
atmospheres of a parameter sweep.  This module holds the host-side pieces:
the split of atmospheres over ranks and the job-wide timing reductions that
bench.py uses; torch.distributed carries them (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations


def shard(items, rank: int, world: int):
    """Round-robin share of `items` for `rank` of `world` (disjoint, covering)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    return list(items)[rank::world]


def shard_indices(n: int, rank: int, world: int):
    return list(range(n))[rank::world]


def max_over_ranks(value: float, device=None) -> float:
    """Largest value over the ranks of the default process group (the job's
    time is the slowest rank's)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_objects(obj):
    """All ranks' objects, in rank order."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out

