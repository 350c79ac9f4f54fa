"""bench.py's multi-GPU path is replicas only: every rank runs the same disk on
its own GPU, the ranks meet at a barrier around the timed region, and the job's
time is the slowest rank's. This checks that host-side logic with two gloo
ranks on the CPU (no GPU, no data-path collective)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    import torch.distributed as dist
    bench.init_replicas()
    bench.replica_barrier(world)
    t, c = bench.replica_reduce(world, 1.0 + rank, 10.0 * (rank + 1))
    out[rank] = (t, c)
    dist.destroy_process_group()


def test_replica_reduce_two_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    # max of the per-rank times, sum of the per-rank eigenvalue counts, seen by every rank
    assert res[0] == res[1] == (2.0, 30.0)


def test_single_rank_is_identity():
    import bench
    assert bench.replica_reduce(1, 3.5, 7.0) == (3.5, 7.0)
