"""Pose sharding across GPUs (one process per GPU, torch.distributed).

Poses, chains and ligand/pocket systems are independent, so the scoring path
shards with no data-path collective: each rank scores its own slice against a
full replica of the pocket and the ligand, and results come back by a host-side
gather.  (The reference's only parallelism is fork-based workers over ligands
and starts, src/lds.ml:2009,2050.)
"""
from __future__ import annotations

import numpy as np


def pose_range(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous, balanced [start, end) slice of n poses for this rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_to_rank0(local: dict, n: int, world: int, rank: int, group=None):
    """Concatenate per-rank result arrays on rank 0 in rank order.

    ``local`` maps names to numpy arrays whose first axis is the rank's slice
    of the n poses.  Returns the full arrays on rank 0 and None elsewhere."""
    import torch.distributed as dist

    if world == 1:
        return local
    parts = [None] * world if rank == 0 else None
    dist.gather_object(local, parts, dst=0, group=group)
    if rank != 0:
        return None
    out = {}
    for k in local:
        out[k] = np.concatenate([p[k] for p in parts], axis=0)
        if out[k].shape[0] != n:
            raise RuntimeError("gathered %d rows of %s, expected %d" % (out[k].shape[0], k, n))
    return out


def max_over_ranks(value: float, group=None) -> float:
    """The slowest rank's time: the job's time under weak scaling."""
    import torch
    import torch.distributed as dist

    if not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    dev = torch.device("cuda", torch.cuda.current_device()) if (
        dist.get_backend(group) == "nccl") else torch.device("cpu")
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
