"""Benchmark: certified interval B&B solves on GB300.

Workload (a step): one complete solve of the n=8 chained-quartic instance
(f = sum p_i (x_{i+1} - x_i^2)^2 + q_i (1 - x_i)^2, p~U[50,150], q~U[0.5,2],
domain [-5,10]^8, 4^8 children per iteration, stop at UB-LB <= 1e-6, seeded).
Metric: child boxes bounded per second.

  value   device time of the persistent solve kernel (CUDA events on the engine
          stream) with the problem already resident on the GPU
  e2e     the same solve through the C ABI call gpugo_solve with host buffers,
          host<->device copies included, wall clock
  cpu_baseline / --impl reference
          the CPU oracle (a C restatement of the reference B&B, OpenMP over the
          children) on the host cores

Multi-GPU: replicas only (one independent solve stream per rank), max time over
ranks, value summed over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "cfg2-chained8: n=8 chained quartic, [-5,10]^8, 4^8 children/iter, S=10, UB-LB<=1e-6"
METRIC = "boxes/s"


# ---------------------------------------------------------------------------
# distributed helpers (replicas only)
# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(backend: str):
    import torch.distributed as dist
    ws, rank, _ = dist_env()
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist if ws > 1 else None


def reduce_max_sum(dist, t_max: float, s_sum: float, device=None):
    """Max of a time and sum of a count over ranks."""
    if dist is None:
        return t_max, s_sum
    import torch
    a = torch.tensor([t_max], dtype=torch.float64, device=device)
    b = torch.tensor([s_sum], dtype=torch.float64, device=device)
    dist.all_reduce(a, op=dist.ReduceOp.MAX)
    dist.all_reduce(b, op=dist.ReduceOp.SUM)
    return float(a.item()), float(b.item())


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits", "-lms", "100"],
                                     stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# FP64 work model of the executed path (used for the roofline numerator)
# ---------------------------------------------------------------------------
# dram__bytes_read.sum + dram__bytes_write.sum of one solve_kernel launch of this
# workload, from an `ncu --set full` capture of `bench.py --steps 2 --warmup 1`
# (its summary is kept under profiles/)
SOLVE_DRAM_BYTES = 226.8e3 + 6.1e3


def fp64_ops_chained(p, iterations: int, bounded: int, sampled: int) -> float:
    """FP64 instructions the chained-family path executes (DADD/DMUL/DFMA/DDIV
    each counted as one; the reference's per-child code list is not re-run).
    Per child: n-1 directed adds (lower-bound chain).  Per sampled child: S(n-1)
    directed adds + S compares.  Per iteration, term tables: (n-1) w^2 (S+1)
    entries x 40 ops and n w^3 gradient entries x 45 ops."""
    n, w, S = p.n, p.wid, p.samples
    per_iter = (n - 1) * w * w * (S + 1) * 40 + n * w ** 3 * 45
    return bounded * (n - 1) + sampled * S * (n - 1 + 1) + iterations * per_iter


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
def run_gpugo(args, dist):
    import torch

    import gpugo_gb300 as G
    from gpugo_gb300 import _lib, problems as P

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    L = _lib.load()
    p = P.config2()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # 256 MiB > 129 MB L2

    eng = G.Engine(max_slots=1, arena_bytes=256 << 20)
    import ctypes
    stats = _lib.Stats()

    def one_step():
        flush.zero_()
        torch.cuda.synchronize()
        t = eng.submit(p, box_cap=4)
        assert t is not None
        eng.run(0)
        _lib.check(L.gpugo_engine_stats(eng._h, ctypes.byref(stats)))
        ms = stats.last_run_ms
        (tk, r), = eng.poll()
        assert r.status == G.CERTIFIED and r.ub - r.lb <= p.gap_tol
        return ms, r

    for _ in range(args.warmup):
        one_step()
    _lib.check(L.gpugo_engine_stats(eng._h, ctypes.byref(stats)))
    launches0 = stats.kernel_launches
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    dev_ms, boxes, sampled, iters = 0.0, 0, 0, 0
    last = None
    for _ in range(args.steps):
        ms, r = one_step()
        dev_ms += ms
        boxes += r.boxes_bounded
        sampled += r.samples_evaluated
        iters += r.iterations
        last = r
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    _lib.check(L.gpugo_engine_stats(eng._h, ctypes.byref(stats)))
    launches = stats.kernel_launches - launches0
    eng.close()
    t_max, boxes_all = reduce_max_sum(dist, dev_ms, float(boxes), device="cuda")

    # end to end through the C ABI (host buffers, copies inside)
    for _ in range(args.warmup):
        G.solve(p, box_cap=4)
    torch.cuda.synchronize()
    e2e_s, e2e_boxes = 0.0, 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = G.solve(p, box_cap=4)
        e2e_s += time.perf_counter() - t0
        e2e_boxes += r.boxes_bounded
    # bytes per step from the raw result struct
    s_spec, keep = G._spec(p)
    res = _lib.Result()
    import numpy as np
    bx = np.zeros((4, 2 * p.n)); lbs = np.zeros(4); xh = np.zeros(p.n)
    dp = ctypes.POINTER(ctypes.c_double)
    _lib.check(L.gpugo_solve(ctypes.byref(s_spec), ctypes.byref(res), bx.ctypes.data_as(dp), lbs.ctypes.data_as(dp),
                             4, xh.ctypes.data_as(dp), None))
    e2e_t, e2e_all = reduce_max_sum(dist, e2e_s, float(e2e_boxes), device="cuda")

    # roofline: FP64 throughput of the persistent kernel against a measured DFMA peak
    peak = ctypes.c_double()
    pms = ctypes.c_double()
    _lib.check(L.gpugo_fp64_peak(5, ctypes.byref(peak), ctypes.byref(pms)))
    ops = fp64_ops_chained(p, iters, boxes, sampled)
    achieved = ops / (dev_ms * 1e-3) / 1e12
    out = {
        "metric": METRIC, "value": boxes_all / (t_max * 1e-3), "unit": "boxes/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded instance, MASTER_SEED+2)",
        "config": {"workload": WORKLOAD, "parallelism": f"replicas{ws}", "l2": "flushed between steps (256 MiB write)",
                   "iterations_per_solve": last.iterations, "boxes_per_solve": last.boxes_bounded,
                   "time_to_certified_ms": t_max / args.steps, "enclosure": [last.lb, last.ub]},
        "e2e": {"value": e2e_all / e2e_t, "unit": "boxes/s", "h2d_bytes_per_step": int(res.h2d_bytes),
                "d2h_bytes_per_step": int(res.d2h_bytes), "ms_per_step": 1e3 * e2e_t / args.steps},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value else None,
                     # DRAM bytes of this launch (read + write) from the committed ncu capture of the
                     # same command: the working set stays in L2
                     "traffic": SOLVE_DRAM_BYTES, "traffic_unit": "bytes per launch (ncu)",
                     "peak_source": "measured in this run: DFMA chains on all SMs (gpugo_fp64_peak), FMA=2 flops",
                     "numerator": "FP64 instructions of the executed path (bench.fp64_ops_chained), as flops"},
        "clocks": clk,
    }
    return out


def run_cpu_baseline(seconds: float = 15.0):
    """The oracle (C restatement of the reference B&B) on the host cores, faithful
    mode (every child's samples evaluated, as the reference does)."""
    import oracle
    from gpugo_gb300 import problems as P
    oracle.build()
    p = P.config2()
    t0 = time.perf_counter()
    boxes = 0
    solves = 0
    while True:
        r = oracle.solve(p, box_cap=4, skip_samples=False)
        boxes += r.boxes_bounded
        solves += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": boxes / dt, "unit": "boxes/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{solves} complete solves of the workload in {dt:.1f} s (OpenMP over children, "
                      f"all sample points evaluated as in the reference)"}, solves, dt


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    import oracle
    from gpugo_gb300 import problems as P
    oracle.build()
    p = P.config2()
    for _ in range(args.warmup):
        oracle.solve(p, box_cap=4, skip_samples=False)
    t0 = time.perf_counter()
    boxes = 0
    for _ in range(args.steps):
        r = oracle.solve(p, box_cap=4, skip_samples=False)
        boxes += r.boxes_bounded
    dt = time.perf_counter() - t0
    v = boxes / dt
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "boxes/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded instance, MASTER_SEED+2)",
            "config": {"workload": WORKLOAD, "parallelism": "host cores"},
            "cpu_baseline": {"value": v, "unit": "boxes/s", "cores": oracle.num_threads(), "kind": "port",
                             "sample": f"{args.steps} complete solves (the reference's Numba CUDA kernels cannot "
                                       f"run here: numba is absent; this is the oracle's C restatement)"},
            "e2e": {"value": v, "unit": "boxes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_batched(args):
    """Config 4: a mixed batch solved by one engine vs the same problems solved
    one per launch (gpugo_solve in a loop); results must be identical."""
    import gpugo_gb300 as G
    from gpugo_gb300 import autotune as A
    from gpugo_gb300 import problems as P
    probs = P.config4(count=args.count)
    tuned = None
    ecfg = A.EngineConfig()
    if args.autotune:
        # block size, candidates per warp and fan-out picked on a sample of the batch;
        # the plain loop then solves the same (re-split) problems
        t0 = time.perf_counter()
        tuned = A.tune(probs, sample=min(512, args.count))
        tune_s = time.perf_counter() - t0
        probs = tuned.apply(probs)
        ecfg = tuned.engine
    for p in probs[:8]:
        G.solve(p, box_cap=4)                      # warm-up
    t0 = time.perf_counter()
    plain = [G.solve(p, box_cap=4) for p in probs]
    t_plain = time.perf_counter() - t0
    dev_plain = sum(r.device_ms for r in plain) * 1e-3
    with G.Engine(max_slots=args.count, arena_bytes=args.arena_gb << 30, threads=ecfg.threads,
                  blocks_per_sm=ecfg.blocks_per_sm, cand_mode=ecfg.cand_mode) as eng:
        eng.solve_all(probs[:8], box_cap=4)        # warm-up
        st0 = eng.stats()
        t0 = time.perf_counter()
        res = eng.solve_all(probs, box_cap=4)
        t_b = time.perf_counter() - t0
        st1 = eng.stats()
    same = all((a.lb, a.ub, a.iterations, a.status) == (b.lb, b.ub, b.iterations, b.status)
               for a, b in zip(plain, res))
    boxes = sum(r.boxes_bounded for r in res)
    return {"metric": "boxes/s", "value": boxes / t_b, "unit": "boxes/s", "n_gpus": 1, "dtype": "f64",
            "higher_is_better": True, "data": "synthetic (config 4 generator, MASTER_SEED+4)",
            "config": {"workload": f"cfg4-batch{args.count}: families F1-F4, n log-uniform 2..64, UB-LB<=1e-6",
                       "certified": sum(r.certified for r in res), "boxes": boxes,
                       "samples_evaluated": sum(r.samples_evaluated for r in res),
                       "max_iterations": max(r.iterations for r in res)},
            "batched_wall_s": t_b, "batched_device_s": (st1["total_run_ms"] - st0["total_run_ms"]) * 1e-3,
            "batched_launches": st1["kernel_launches"] - st0["kernel_launches"],
            "plain_wall_s": t_plain, "plain_device_s": dev_plain, "plain_launches": 2 * len(probs),
            "speedup_vs_plain": t_plain / t_b, "identical_to_plain": same,
            "engine": ecfg.label(),
            **({"autotune": {"seconds": tune_s, "fanout": {f"{lo}-{hi}": list(v) for (lo, hi), v in
                                                             tuned.fanout.items()},
                             "trials": tuned.trials}} if tuned else {})}


def run_serving(args):
    """Config 5: Poisson stream of requests, continuous batching, p50/p99."""
    import gpugo_gb300 as G
    from gpugo_gb300 import autotune as A
    from gpugo_gb300 import problems as P
    from gpugo_gb300.serve import serve
    stream = P.config5(count=args.count, rate=args.rate)
    ecfg, tuned, tune_s = A.EngineConfig(), None, 0.0
    if args.autotune:
        # tuned on a sample of the request mix before the stream starts
        t0 = time.perf_counter()
        tuned = A.tune([p for _, p in stream], sample=min(128, args.count))
        tune_s = time.perf_counter() - t0
        stream = list(zip([t for t, _ in stream], tuned.apply([p for _, p in stream])))
        ecfg = tuned.engine
    slots = min(args.count, 2048)
    with G.Engine(max_slots=slots, arena_bytes=args.arena_gb << 30, threads=ecfg.threads,
                  blocks_per_sm=ecfg.blocks_per_sm, cand_mode=ecfg.cand_mode) as eng:
        rep = serve(stream, max_slots=slots, slice_iters=args.slice, engine=eng)
    sm = rep.summary()
    return {"metric": "time-to-certified p50/p99 (ms) and boxes/s", "value": sm["boxes_per_s"], "unit": "boxes/s",
            "p50_ms": sm["p50_ms"], "p99_ms": sm["p99_ms"], "n_gpus": 1, "dtype": "f64",
            "data": "synthetic (config 5 generator, MASTER_SEED+5)",
            "config": {"workload": f"cfg5-serve{args.count}: Poisson {args.rate}/s, F1-F4, n log-uniform 2..128, "
                                   f"tol 1e-6 or 1e-4, pool arena {args.arena_gb} GiB",
                       "slice_iters": args.slice, "engine": ecfg.label(),
                       **({"autotune_s": tune_s, "fanout": {f"{lo}-{hi}": list(v) for (lo, hi), v in
                                                             tuned.fanout.items()}} if tuned else {})},
            **{k: v for k, v in sm.items() if k not in ("p50_ms", "p99_ms")}}


def run_list_pass(args):
    """The grid-wide list pass on large lists: the 50-variable Rastrigin script's
    loop (4^10 children per iteration, rastrigin50.py:844-1289) for a few
    iterations; the list grows by about 1 Mi entries per iteration.  The pass
    is timed with the engine's phase stamps (GPUGO_PHASE_STAMPS) and its
    algorithmic bytes are 16 B per entry read plus 16 B per entry written."""
    import os
    import tempfile
    import numpy as np
    path = os.path.join(tempfile.mkdtemp(), "stamps")
    os.environ["GPUGO_PHASE_STAMPS"] = path
    import gpugo_gb300 as G
    from gpugo_gb300 import problems as P
    n = 50
    p = P.Problem(P.COSQUAD, n, np.tile([-5.5, 6.0], n), np.concatenate([np.ones(n), np.full(n, 10.0), np.ones(n)]),
                  wid=4, group=10, samples=10, stop_mode=P.STOP_WIDTH, width_tol=1e-4, ub_init=1e6,
                  max_iter=args.steps, pool_cap=1 << 26)
    with G.Engine(max_slots=1, arena_bytes=8 << 30) as eng:
        eng.submit(p, box_cap=4, trace_cap=4096)
        eng.run(0)
        (_, r), = eng.poll()
    rows = open(path).read().strip().split("run ")[-1].split("\n")[1:]
    st = np.array([[int(x) for x in l.split()] for l in rows], dtype=np.float64)
    per = []
    for it in range(st.shape[0]):
        if st[it, 3] <= 0:
            continue
        us = (st[it, 3] - st[it, 2]) / 1e3
        n_in = (r.trace["pool"][it - 1] if it > 0 else 0) + r.trace["n_surv"][it]
        n_out = r.trace["pool"][it]
        per.append({"iteration": it, "entries_in": int(n_in), "entries_out": int(n_out), "us": round(us, 1),
                    "GBps": round((n_in + n_out) * 16 / (us * 1e-6) / 1e9, 1)})
    big = [d for d in per if d["entries_in"] >= (1 << 20) and d["entries_out"] >= (1 << 20)]
    best = max(big, key=lambda d: d["GBps"]) if big else None
    return {"metric": "list pass GB/s (algorithmic)", "value": best["GBps"] if best else None, "unit": "GB/s",
            "n_gpus": 1, "dtype": "f64/u64", "config": {"workload": "rastrigin50 reference loop, 4^10 children/iter",
                                                      "iterations": int(st.shape[0])},
            "per_iteration": per}


def run_single(args):
    import gpugo_gb300 as G
    from gpugo_gb300 import problems as P
    p = {"cfg1": P.config1, "cfg3": lambda: P.config3(split=(3, 8))}[args.workload]()
    for _ in range(args.warmup):
        G.solve(p, box_cap=4)
    dev, boxes = 0.0, 0
    for _ in range(args.steps):
        r = G.solve(p, box_cap=4)
        dev += r.device_ms
        boxes += r.boxes_bounded
    return {"metric": "boxes/s", "value": boxes / (dev * 1e-3), "unit": "boxes/s", "n_gpus": 1, "dtype": "f64",
            "steps": args.steps, "ms_per_step": dev / args.steps,
            "config": {"workload": p.tag, "n": p.n, "split": [p.wid, p.group], "iterations": r.iterations,
                       "boxes_per_solve": r.boxes_bounded, "enclosure": [r.lb, r.ub], "certified": r.certified}}


def run_codelist(args):
    """The reference's seven benchmarks without a built-in family, as code
    lists (n = 8, split 3^8, UB-LB <= 1e-6), plus config 2 restated as a code
    list next to its built-in kernel; the CPU oracle solves each once."""
    import time
    import gpugo_gb300 as G
    import oracle
    from gpugo_gb300 import objectives as O
    from gpugo_gb300 import problems as P
    oracle.build()
    cases = [(name, O.problem(name, 8, tol=1e-6)) for name in sorted(O.REFERENCE)]
    cases += [("chained8-builtin", P.config2()), ("chained8-codelist", O.as_codelist(P.config2()))]
    rows, dev_tot, boxes_tot = {}, 0.0, 0
    cpu_s, cpu_boxes = 0.0, 0
    for name, p in cases:
        for _ in range(args.warmup):
            G.solve(p, box_cap=4)
        ms = []
        for _ in range(args.steps):
            r = G.solve(p, box_cap=4)
            ms.append(r.device_ms)
        ms.sort()
        dev_tot += sum(ms)
        boxes_tot += r.boxes_bounded * len(ms)
        t0 = time.perf_counter()
        ro = oracle.solve(p, box_cap=4, skip_samples=False)
        dt = time.perf_counter() - t0
        assert (ro.lb, ro.ub, ro.iterations) == (r.lb, r.ub, r.iterations), name
        if not name.startswith("chained8"):
            cpu_s += dt
            cpu_boxes += ro.boxes_bounded
        rows[name] = {"ms_median": round(ms[len(ms) // 2], 4), "iterations": r.iterations,
                      "boxes": r.boxes_bounded, "certified": r.certified, "enclosure": [r.lb, r.ub],
                      "cpu_oracle_ms": round(dt * 1e3, 2)}
    return {"metric": "boxes/s (code-list objectives)", "value": boxes_tot / (dev_tot * 1e-3), "unit": "boxes/s",
            "n_gpus": 1, "dtype": "f64", "steps": args.steps,
            "config": {"workload": "seven reference benchmarks as code lists, n=8, split 3^8, UB-LB<=1e-6; "
                                   "config 2 built-in vs code list", "per_objective": rows},
            "cpu_baseline": {"value": cpu_boxes / cpu_s, "unit": "boxes/s", "cores": oracle.num_threads(),
                             "kind": "port", "sample": "one oracle solve of each of the seven objectives"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpugo", choices=["gpugo", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--workload", default="cfg2",
                    choices=["cfg2", "cfg1", "cfg3", "cfg4", "cfg5", "listpass", "codelist"],
                    help="cfg2 is the benchmark line; the others print their own records")
    ap.add_argument("--count", type=int, default=None, help="instances (cfg4: 1024) or requests (cfg5: 4096)")
    ap.add_argument("--rate", type=float, default=20000.0)
    ap.add_argument("--slice", type=int, default=16)
    ap.add_argument("--arena-gb", type=int, default=80)
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="cfg4/cfg5: skip the autotuner (block size, candidates per warp, fan-out)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.count is None:
        args.count = 4096 if args.workload == "cfg5" else 1024
    ws, rank, local = dist_env()
    if args.workload != "cfg2" and args.impl == "gpugo":
        fn = {"cfg1": run_single, "cfg3": run_single, "cfg4": run_batched, "cfg5": run_serving,
              "listpass": run_list_pass, "codelist": run_codelist}[args.workload]
        print(json.dumps(fn(args)))
        return
    if args.impl == "reference":
        out = run_reference(args)
        if out is not None:
            print(json.dumps(out))
        return
    dist = init_dist("nccl")
    out = run_gpugo(args, dist)
    if rank == 0:
        cb, _, _ = run_cpu_baseline(args.cpu_seconds)
        out["cpu_baseline"] = cb
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
