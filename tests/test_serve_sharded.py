"""Serving across GPUs, host side: the arrivals are dealt round-robin over the
ranks (one process and one engine per GPU), each rank serves its share, and
rank 0 merges the latencies into one p50/p99 and the boxes into one rate.
Two gloo ranks on the CPU with a fake engine (no GPU); unmeasured on hardware
until several GPUs are available to one run."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from gpugo_gb300 import problems as P
from gpugo_gb300.serve import merge_records, partition_stream


def _stream(k):
    return [(0.0002 * i, P.instance(P.COSQUAD, 2, i, tag=f"q{i}")) for i in range(k)]


def test_partition_is_round_robin_and_complete():
    s = _stream(11)
    parts = [partition_stream(s, r, 3) for r in range(3)]
    assert [len(p) for p in parts] == [4, 4, 3]
    assert [q.tag for _, q in parts[1]] == ["q1", "q4", "q7", "q10"]
    tags = sorted(q.tag for part in parts for _, q in part)
    assert tags == sorted(q.tag for _, q in s)
    assert partition_stream(s, 0, 1) == s
    with pytest.raises(ValueError):
        partition_stream(s, 3, 3)


def test_merge_takes_percentiles_over_all_requests():
    a = {"latencies_ms": [1.0, 2.0, 3.0], "boxes": 30, "certified": 3, "rejected": 0, "requests": 3,
         "wall_s": 2.0, "device_s": 1.0, "launches": 4}
    b = {"latencies_ms": [10.0, 20.0], "boxes": 20, "certified": 2, "rejected": 1, "requests": 3,
         "wall_s": 4.0, "device_s": 3.0, "launches": 2}
    m = merge_records([a, b])
    lat = [1.0, 2.0, 3.0, 10.0, 20.0]
    assert m["p50_ms"] == float(np.percentile(lat, 50)) and m["p99_ms"] == float(np.percentile(lat, 99))
    assert (m["requests"], m["certified"], m["rejected"], m["boxes"]) == (6, 5, 1, 50)
    assert m["wall_s"] == 4.0 and m["boxes_per_s"] == 50 / 4.0 and m["ranks"] == 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from test_serve_host import FakeEngine
    from gpugo_gb300.serve import serve_sharded
    dist.init_process_group("gloo")
    eng = FakeEngine(slots=4, iters=1 + rank)        # rank 1 is slower: two runs per solve
    merged = serve_sharded(_stream(21), dist, max_slots=4, slice_iters=1, engine=eng)
    out[rank] = (merged, list(eng.admit_order))
    dist.destroy_process_group()


def test_two_ranks_serve_their_shares_and_rank0_merges():
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    merged, order0 = out[0]
    none, order1 = out[1]
    assert none is None
    assert order0 == [f"q{i}" for i in range(0, 21, 2)]
    assert order1 == [f"q{i}" for i in range(1, 21, 2)]
    assert merged["ranks"] == 2 and merged["requests"] == 21 and merged["certified"] == 21
    assert merged["boxes"] == 210 and merged["rejected"] == 0
    assert 0 < merged["p50_ms"] <= merged["p99_ms"]
