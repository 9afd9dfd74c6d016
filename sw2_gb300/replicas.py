"""Replica runs over several GPUs of one node (one process per GPU).

The step does not shard: each rank advances its own independent case (its
own seed) and no data crosses ranks. The only collectives are for timing:
a barrier around the timed region and, afterwards, the slowest rank's time
and the total work, from which the whole-job throughput follows.
"""
from __future__ import annotations

import os


def dist_env():
    """(world size, rank, local rank) from the torchrun environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate(cell_updates: float, seconds: float, device=None):
    """Whole-job throughput of one timed region: (total cell-updates over all
    ranks) / (slowest rank's seconds). Returns (throughput, total, max seconds).
    Without an initialised process group it is the local figure."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return cell_updates / seconds, cell_updates, seconds
    dev = device if device is not None else "cpu"
    work = torch.tensor([float(cell_updates)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(work, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total, tmax = float(work.item()), float(t.item())
    return total / tmax, total, tmax
