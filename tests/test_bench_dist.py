"""bench.py's multi-GPU path is replicas only: each rank solves its own stream,
the time is the max over ranks and the work the sum.  This runs the aggregation
with two gloo ranks on the CPU (the GPU step itself is covered by the GPU tests)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist = bench.init_dist("gloo")
    ws, r, local = bench.dist_env()
    t, s = bench.reduce_max_sum(dist, 10.0 + rank, 100.0 * (rank + 1), device="cpu")
    out[rank] = (ws, r, t, s)
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == (2, 0, 11.0, 300.0)
    assert out[1] == (2, 1, 11.0, 300.0)


def test_single_rank_is_identity():
    import bench
    assert bench.reduce_max_sum(None, 3.0, 7.0) == (3.0, 7.0)
