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


def test_gpus_flag_must_match_the_launched_ranks(monkeypatch):
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    bench.check_gpus(1)
    with pytest.raises(SystemExit):
        bench.check_gpus(8)               # one process does not stand in for eight GPUs
    monkeypatch.setenv("WORLD_SIZE", "2")
    bench.check_gpus(2)
    with pytest.raises(SystemExit):
        bench.check_gpus(1)


def test_counter_profile_is_parsed(tmp_path):
    import bench
    f = tmp_path / "p.md"
    f.write_text("# x\n\n    fp64_thread_ops_per_box: 1234.5\n    dram_bytes_per_box: 6.5e1\nother: 3\n")
    c = bench.profile_counters(str(f))
    assert c == {"fp64_thread_ops_per_box": 1234.5, "dram_bytes_per_box": 65.0}
    assert bench.profile_counters(str(tmp_path / "absent.md")) is None


def test_batch_problems_are_the_same_in_every_arm():
    """The GPU arm, the plain loop and both CPU legs solve one list of problems:
    the generator and the fan-out table are deterministic."""
    import bench
    a, b = bench.batch_problems(64), bench.batch_problems(64)
    assert [(p.family, p.n, p.wid, p.group, p.gap_tol) for p in a] == \
        [(p.family, p.n, p.wid, p.group, p.gap_tol) for p in b]
    assert all((p.coef == q.coef).all() and (p.domain == q.domain).all() for p, q in zip(a, b))
    assert all((p.wid, p.group) == ((3, 5) if p.n <= 16 else (3, 6)) for p in a if p.n >= 8)
    s = bench.cpu_sample(a, 16)
    assert len(s) == 16 and s[0] is a[0] and s[1] is a[4]


def test_reference_flop_count():
    import bench
    from gpugo_gb300 import problems as P
    p = P.config2()       # chained quartic, n = 8, S = 10
    assert bench.reference_flops(p, 1, 0) == 18 * 7 * 11
    assert bench.reference_flops(p, 2, 1) == 2 * 18 * 7 * 11 + 26 * 8
