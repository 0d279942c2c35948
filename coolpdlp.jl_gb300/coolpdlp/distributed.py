"""Several GPUs, one process each (torchrun): which LPs a rank solves and how
the ranks' timings combine.

A single LP does not shard (each half-step would need an all-gather of the
iterate), so single-LP runs on N GPUs are N replicas.  Batched and served LPs
are independent units: rank r of N takes the LPs whose index is r mod N, solves
them on its own GPU with no collective on the data path, and only the
timings are reduced (the slowest rank's time over all ranks' LPs).
"""
from __future__ import annotations

import os


def dist_info():
    """(world_size, rank, local_rank) from the torchrun environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def shard_indices(count: int, rank: int, world: int) -> list:
    """The LP indices rank `rank` of `world` solves: every world-th from rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(range(rank, int(count), world))


def reduce_over_ranks(value: float, op: str = "max", device=None) -> float:
    """max / sum of a per-rank scalar over the process group (no group, or a
    world of one: the value itself).  Uses the group's backend (NCCL with a
    CUDA device, gloo on the CPU)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())
