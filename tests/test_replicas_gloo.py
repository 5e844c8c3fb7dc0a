"""Replica logic of the multi-rank benchmark on CPU: two gloo ranks.

Each rank takes its share of the points, times its own work, and rank 0 gets
the maximum over ranks; shares tile the point range exactly.
"""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from smolyax_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_points, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    w, r, lr = replicas.init("gloo")
    assert (w, r, lr) == (world, rank, rank)
    start, stop = replicas.shard(n_points, w, r)
    replicas.barrier()
    local = [float(stop - start), 10.0 * (rank + 1)]  # this rank's "timings"
    mx = replicas.max_over_ranks(local)
    out[rank] = (start, stop, mx)
    dist.destroy_process_group()


@pytest.mark.parametrize("n_points", [10, 100_001])
def test_two_gloo_ranks(n_points):
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_worker, args=(world, _free_port(), n_points, out), nprocs=world, join=True,
                       start_method="spawn")
    spans = sorted((out[r][0], out[r][1]) for r in range(world))
    assert spans[0][0] == 0 and spans[-1][1] == n_points
    assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    for r in range(world):
        assert out[r][2][1] == 10.0 * world  # max over ranks seen by every rank
        assert out[r][2][0] == float(max(b - a for a, b in spans))


def test_shard_single_and_errors():
    assert replicas.shard(7, 1, 0) == (0, 7)
    assert [replicas.shard(7, 3, r) for r in range(3)] == [(0, 3), (3, 5), (5, 7)]
    with pytest.raises(ValueError):
        replicas.shard(7, 2, 2)
    assert replicas.max_over_ranks([1.5, 2.0]) == [1.5, 2.0]
