"""One process per GPU, each evaluating its own query points.

Query points are independent and a built interpolant is small, so the
evaluation path shards by points with no exchange step: every rank holds a
full copy of the interpolant (a replica) and evaluates its own batch.  The
only cross-rank operations are a barrier around timed regions and the maximum
of the per-rank timings.  Ranks read RANK / LOCAL_RANK / WORLD_SIZE (and
MASTER_ADDR / MASTER_PORT for the rendezvous) from the environment, as set by
``torch.distributed.run``.
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


def rank_info():
    """(world_size, rank, local_rank) from the launcher's environment."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init(backend: str = "nccl"):
    """Join the process group when more than one rank runs; returns rank_info()."""
    world, rank, local = rank_info()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend)
    return world, rank, local


def shard(n_points: int, world: int, rank: int):
    """[start, stop) of this rank's share of n_points (contiguous, sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world of size %d" % (rank, world))
    base, extra = divmod(int(n_points), world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def barrier(device=None):
    """Barrier across ranks (if any), then wait for this rank's device work."""
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
    if device is not None and torch.device(device).type == "cuda":
        torch.cuda.synchronize(device)


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of a list of floats over all ranks."""
    vals = [float(v) for v in values]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return vals
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]
