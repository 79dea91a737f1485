"""Benchmark: certified interval B&B solves on GB300.

Workload (a step, the default line): one certified solve of the whole mixed
batch of 1024 instances -- families F1-F4 (cosine-quadratic, chained quartic,
exp-sqrt composite, product-cosine), n log-uniform in 2..64, stop at
UB-LB <= 1e-6, seeded -- in one persistent engine.  Metric: child boxes bounded
per second.

  value   device time of the engine's persistent kernel (CUDA events on the
          engine stream) with the problems admitted
  e2e     the same batch through the public API (Engine.solve_all: problem
          descriptions from host memory, results and minimiser boxes back to
          host memory), wall clock, copies included
  config  the plain one-instance-per-launch path on the same problems
          (gpugo_solve in a loop: time, speed-up, identical results) and a
          serving record: the 4096-request Poisson stream, p50/p99 latency
  cpu_baseline / --impl reference
          the CPU oracle (a C restatement of the reference B&B, OpenMP over the
          children) on the host cores, on instances of the same batch

Multi-GPU: replicas (one batch per rank; max time over ranks, boxes summed);
the serving record deals the arrivals round-robin over the ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("cfg4-batch1024: 1024 mixed instances (F1-F4, n log-uniform 2..64), UB-LB<=1e-6, "
            "one persistent engine")
METRIC = "boxes/s"
# ncu summary of this workload's persistent kernel (FP64 instruction and DRAM counters)
COUNTER_PROFILE = os.path.join(ROOT, "profiles", "solve_kernel_cfg4_batch1024.md")


# ---------------------------------------------------------------------------
# distributed helpers (replicas only)
# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def check_gpus(requested: int) -> None:
    """--gpus N must match the ranks the launcher started (torchrun sets
    WORLD_SIZE); a single process never stands in for several GPUs."""
    ws, _, _ = dist_env()
    if requested != ws:
        raise SystemExit(f"bench.py --gpus {requested} but WORLD_SIZE={ws}: launch N ranks with "
                         f"python -m torch.distributed.run --nproc-per-node {requested} bench.py --gpus {requested}")


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
# workload and work counts
# ---------------------------------------------------------------------------
def batch_problems(count: int = 1024):
    """The mixed batch with the tuned fan-out table applied: every arm of the
    benchmark (GPU batch, plain loop, CPU oracle) solves these same problems."""
    from gpugo_gb300 import autotune as A
    from gpugo_gb300 import problems as P
    return A.apply_fanout(P.config4(count=count))


def serving_stream(count: int, rate: float):
    from gpugo_gb300 import autotune as A
    from gpugo_gb300 import problems as P
    stream = P.config5(count=count, rate=rate)
    return list(zip([t for t, _ in stream], A.apply_fanout([p for _, p in stream])))


def cpu_sample(probs, k: int):
    """Every (len/k)-th instance of the batch: the CPU legs' bounded sample."""
    from gpugo_gb300 import autotune as A
    return A.sample_problems(probs, k)


T_TRANS = 20   # FP64 operations charged per transcendental endpoint evaluation (declared convention)


def reference_flops(p, boxes: int, sampled: int) -> float:
    """Interval FP64 operations the reference's code lists spend on `boxes`
    children, `sampled` of which also reach the derivative list: per child the
    value list and S sample lists, per sampled child the gradient list, with the
    per-operation weights add/times 2, multiply 8, square 2, transcendental T."""
    n, S, T = p.n, p.samples, T_TRANS
    fam = int(p.family)
    if fam == 1:
        per, grad = n * (10 + 2 * T), n * (8 + 2 * T)
    elif fam == 2:
        per, grad = 18 * (n - 1), 26 * n
    elif fam == 3:
        per, grad = n * (10 + 2 * T) + 4 * T + 14, n * (30 + 4 * T)
    else:
        per, grad = n * (14 + 2 * T) + 6, n * (38 + 6 * T)
    return float(boxes) * per * (1 + S) + float(sampled) * grad


def profile_counters(path: str = COUNTER_PROFILE) -> dict | None:
    """Per-box FP64 and DRAM figures of this workload's persistent kernel from
    its ncu summary (lines `key: value` in the summary's counter block)."""
    if not os.path.exists(path):
        return None
    out = {}
    for line in open(path):
        m = re.match(r"^\s*(fp64_thread_ops_per_box|dram_bytes_per_box|boxes_captured|fp64_pipe_active_pct)"
                     r":\s*([0-9.eE+-]+)", line)
        if m:
            out[m.group(1)] = float(m.group(2))
    return out or None


# ---------------------------------------------------------------------------
# GPU arm: the batch line
# ---------------------------------------------------------------------------
def tune_engine(probs, args):
    """Block size and candidate scheduling picked on half the batch (work-neutral:
    the results are identical under every configuration)."""
    from gpugo_gb300 import autotune as A
    if not args.autotune:
        return A.EngineConfig(), 0.0, []
    t0 = time.perf_counter()
    tr = A.tune(probs, sample=min(512, len(probs)), fanout_options=(), n_classes=(),
                timer=lambda ps, cfg: A.time_engine(ps, cfg, arena_bytes=args.arena_gb << 30))
    return tr.engine, time.perf_counter() - t0, tr.trials


def run_batch(args, dist):
    import ctypes

    import torch

    import gpugo_gb300 as G
    from gpugo_gb300 import _lib
    from gpugo_gb300.serve import serve_sharded

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    L = _lib.load()
    probs = batch_problems(args.count)
    ecfg, tune_s, trials = tune_engine(probs, args)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # 256 MiB > 129 MB L2

    eng = G.Engine(max_slots=len(probs), arena_bytes=args.arena_gb << 30, threads=ecfg.threads,
                   blocks_per_sm=ecfg.blocks_per_sm, cand_mode=ecfg.cand_mode)
    for _ in range(args.warmup):
        eng.solve_all(probs, box_cap=4)
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    dev_ms, wall_s, boxes, sampled = 0.0, 0.0, 0, 0
    st_first = eng.stats()
    res = None
    for _ in range(args.steps):
        flush.zero_()                      # L2 flushed between steps, outside both clocks
        torch.cuda.synchronize()
        st0 = eng.stats()
        t0 = time.perf_counter()
        res = eng.solve_all(probs, box_cap=4)
        wall_s += time.perf_counter() - t0
        st1 = eng.stats()
        dev_ms += st1["total_run_ms"] - st0["total_run_ms"]
        boxes += sum(r.boxes_bounded for r in res)
        sampled += sum(r.samples_evaluated for r in res)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    st_last = eng.stats()
    eng.close()
    assert all(r.certified and r.ub - r.lb <= p.gap_tol for r, p in zip(res, probs))
    launches = st_last["kernel_launches"] - st_first["kernel_launches"]
    h2d = (st_last["h2d_bytes"] - st_first["h2d_bytes"]) // args.steps
    d2h = (st_last["d2h_bytes"] - st_first["d2h_bytes"]) // args.steps
    t_max, boxes_all = reduce_max_sum(dist, dev_ms, float(boxes), device="cuda")
    w_max, _ = reduce_max_sum(dist, wall_s, 0.0, device="cuda")

    # the plain path: the same problems, one gpugo_solve (one launch series) each
    batch_s = wall_s / args.steps
    plain_s = plain_dev_s = same = None
    if args.plain:
        for p in probs[:8]:
            G.solve(p, box_cap=4)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plain = [G.solve(p, box_cap=4) for p in probs]
        plain_s = time.perf_counter() - t0
        plain_dev_s = sum(r.device_ms for r in plain) * 1e-3
        same = all((a.lb, a.ub, a.iterations, a.boxes_bounded, a.status) ==
                   (b.lb, b.ub, b.iterations, b.boxes_bounded, b.status) for a, b in zip(plain, res))

    # serving: the config-5 stream, arrivals dealt over the ranks
    serving = None
    if args.serve_count > 0:
        stream = serving_stream(args.serve_count, args.rate)
        slots = min(len(stream), 2048)
        with G.Engine(max_slots=slots, arena_bytes=args.arena_gb << 30, threads=ecfg.threads,
                      blocks_per_sm=ecfg.blocks_per_sm, cand_mode=ecfg.cand_mode) as seng:
            serving = serve_sharded(stream, dist, max_slots=slots, slice_iters=args.slice, engine=seng,
                                    order=args.serve_order)
        if serving is not None:
            serving["workload"] = (f"cfg5-serve{args.serve_count}: Poisson {args.rate:g}/s, F1-F4, n log-uniform "
                                   f"2..128, tol 1e-6 or 1e-4, arena {args.arena_gb} GiB, slice {args.slice}, "
                                   f"admission by {args.serve_order}")

    # roofline: FP64 throughput of the persistent kernel against a DFMA peak measured now
    peak = ctypes.c_double()
    pms = ctypes.c_double()
    _lib.check(L.gpugo_fp64_peak(5, ctypes.byref(peak), ctypes.byref(pms)))
    cnt = profile_counters()
    sec = dev_ms * 1e-3
    ref_fl = sum(reference_flops(p, r.boxes_bounded, r.samples_evaluated) for p, r in zip(probs, res)) * args.steps
    roof = {"bound": "fp64", "peak": peak.value, "unit": "TFLOP/s",
            "peak_source": "measured in this run: DFMA chains on all SMs (gpugo_fp64_peak), FMA = 2 flops; "
                           "MEASURED_PEAKS.json has no FP64 figure",
            "reference_equivalent_tflops": ref_fl / sec / 1e12,
            "reference_equivalent_note": "the reference's per-child code-list work (value + S samples + gradient, "
                                         f"add 2, mul 8, transcendental {T_TRANS}) over the same boxes: term tables "
                                         "and sample skipping remove most of it with identical results"}
    if cnt and cnt.get("fp64_thread_ops_per_box"):
        ach = cnt["fp64_thread_ops_per_box"] * boxes / sec / 1e12
        roof.update({"achieved": ach, "frac": ach / peak.value if peak.value else None,
                     "numerator": "executed FP64 thread operations (DADD, DMUL = 1, DFMA = 2) per bounded box "
                                  "from ncu's sm__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum over "
                                  "this workload's kernel, times the boxes of this run",
                     "traffic": cnt.get("dram_bytes_per_box", 0.0) * boxes / args.steps,
                     "traffic_unit": "DRAM bytes per step (ncu dram__bytes_read.sum + write.sum per box x boxes)",
                     "counter_source": os.path.relpath(COUNTER_PROFILE, ROOT)})
    else:
        roof.update({"achieved": None, "frac": None, "traffic": None})

    out = {
        "metric": METRIC, "value": boxes_all / (t_max * 1e-3), "unit": "boxes/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded instances, config-4 and config-5 generators)",
        "config": {"workload": WORKLOAD, "parallelism": f"replicas{ws}",
                   "l2": "flushed between steps (256 MiB write)",
                   "engine": ecfg.label(), "engine_tuning_s": tune_s,
                   "engine_trials": [{"config": t["config"], "seconds": round(t["seconds"], 4)} for t in trials],
                   "fanout": "the autotuner's table: 3^5 children per iteration for n = 5 and n in 8..16, 3^6 "
                             "for n = 6 and above 16, 3^7 for n = 7, 7^4 / 9^3 / 31^2 for n = 4 / 3 / 2",
                   "instances": len(probs), "certified": sum(r.certified for r in res),
                   "boxes_per_step": boxes // args.steps, "samples_per_step": sampled // args.steps,
                   "iterations_max": max(r.iterations for r in res),
                   "time_to_certified_batch_ms": t_max / args.steps,
                   "batch_wall_s": batch_s,
                   "plain_wall_s": plain_s, "plain_device_s": plain_dev_s, "plain_launch_series": len(probs),
                   "speedup_vs_plain": plain_s / batch_s if plain_s else None,
                   "speedup_vs_plain_device": plain_dev_s / (sec / args.steps) if plain_dev_s else None,
                   "identical_to_plain": same,
                   "serving": serving},
        "e2e": {"value": boxes_all / w_max, "unit": "boxes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * w_max / args.steps,
                "api": "Engine.solve_all (gpugo_submit_batch / gpugo_run / gpugo_poll), host buffers"},
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clk,
    }
    return out


# ---------------------------------------------------------------------------
# CPU legs
# ---------------------------------------------------------------------------
def run_cpu_baseline(probs, k: int = 16):
    """The oracle on every (1024/k)-th instance of the batch: once as the
    reference computes (every child's samples evaluated), once with the GPU's
    sample skipping (children whose LB is above the UB keep their samples
    unevaluated; same results)."""
    import oracle
    oracle.build()
    samp = cpu_sample(probs, k)
    out = {}
    for skip in (False, True):
        t0 = time.perf_counter()
        boxes = 0
        for p in samp:
            boxes += oracle.solve(p, box_cap=4, skip_samples=skip).boxes_bounded
        dt = time.perf_counter() - t0
        out[skip] = (boxes / dt, dt)
    (v, dt), (v2, dt2) = out[False], out[True]
    return {"value": v, "unit": "boxes/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{len(samp)} of the {len(probs)} batch instances (every {len(probs) // len(samp)}th), "
                      f"complete solves in {dt:.1f} s, OpenMP over the children, every child's samples evaluated "
                      f"as in the reference",
            "skip_samples_value": v2,
            "skip_samples_note": f"the same {len(samp)} solves with the GPU's sample skipping: {dt2:.1f} s"}


def run_reference(args):
    """--impl reference: the reference's B&B on the host cores.  The reference's
    own code is Numba CUDA and cannot run on this machine; the oracle (a C
    restatement of its algorithm, OpenMP over the children, every child's
    samples evaluated) stands in.  Each step solves 4 instances of the batch,
    the steps walking through a 64-instance sample (every 16th instance)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    import oracle
    oracle.build()
    probs = batch_problems(args.count)
    samp = cpu_sample(probs, 64)
    per = 4
    small = min(samp, key=lambda p: p.n)
    for _ in range(args.warmup):
        oracle.solve(small, box_cap=4, skip_samples=False)
    t0 = time.perf_counter()
    boxes = 0
    for k in range(args.steps):
        for j in range(per):
            boxes += oracle.solve(samp[(k * per + j) % len(samp)], box_cap=4, skip_samples=False).boxes_bounded
    dt = time.perf_counter() - t0
    v = boxes / dt
    sample = (f"{args.steps} steps of {per} complete solves each, walking through {len(samp)} of the "
              f"{len(probs)} batch instances (every {len(probs) // len(samp)}th); the reference's Numba CUDA "
              f"kernels cannot run here (numba is absent), so this is the oracle's C restatement of its B&B")
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "boxes/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded instances, config-4 generator)",
            "config": {"workload": WORKLOAD, "parallelism": "host cores"},
            "cpu_baseline": {"value": v, "unit": "boxes/s", "cores": oracle.num_threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "boxes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# other workloads (their own records)
# ---------------------------------------------------------------------------
def run_chained8(args):
    """Config 2: one certified solve of the n=8 chained quartic (4^8 children per
    iteration) per step, resident (engine CUDA events) and through gpugo_solve."""
    import ctypes

    import numpy as np
    import torch

    import gpugo_gb300 as G
    from gpugo_gb300 import _lib, problems as P
    L = _lib.load()
    p = P.config2()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    eng = G.Engine(max_slots=1, arena_bytes=256 << 20)

    def one_step():
        flush.zero_()
        torch.cuda.synchronize()
        assert eng.submit(p, box_cap=4) is not None
        eng.run(0)
        ms = eng.stats()["last_run_ms"]
        (tk, r), = eng.poll()
        assert r.status == G.CERTIFIED and r.ub - r.lb <= p.gap_tol
        return ms, r

    for _ in range(args.warmup):
        one_step()
    dev_ms, boxes = 0.0, 0
    for _ in range(args.steps):
        ms, r = one_step()
        dev_ms += ms
        boxes += r.boxes_bounded
    eng.close()
    for _ in range(args.warmup):
        G.solve(p, box_cap=4)
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        G.solve(p, box_cap=4)
        e2e_s += time.perf_counter() - t0
    peak = ctypes.c_double()
    pms = ctypes.c_double()
    _lib.check(L.gpugo_fp64_peak(5, ctypes.byref(peak), ctypes.byref(pms)))
    return {"metric": METRIC, "value": boxes / (dev_ms * 1e-3), "unit": "boxes/s", "n_gpus": 1, "dtype": "f64",
            "steps": args.steps, "ms_per_step": dev_ms / args.steps,
            "config": {"workload": "cfg2-chained8: n=8 chained quartic, [-5,10]^8, 4^8 children/iter, S=10, "
                                   "UB-LB<=1e-6", "iterations": r.iterations, "boxes_per_solve": r.boxes_bounded,
                       "enclosure": [r.lb, r.ub]},
            "e2e": {"value": boxes / e2e_s, "unit": "boxes/s", "ms_per_step": 1e3 * e2e_s / args.steps},
            "fp64_peak_tflops": peak.value}


def run_batched(args):
    """Config 4 with the full autotuner (engine configuration and fan-out tuned
    on the batch), against the plain kernel on the same re-split problems."""
    import gpugo_gb300 as G
    from gpugo_gb300 import autotune as A
    from gpugo_gb300 import problems as P
    probs = P.config4(count=args.count)
    t0 = time.perf_counter()
    tuned = A.tune(probs, sample=min(512, args.count), n_classes=tuple(A.SMALL_FANOUT) + A.N_CLASSES,
                   fanout_options=dict(A.SMALL_FANOUT), per_class=32,
                   timer=lambda ps, cfg: A.time_engine(ps, cfg, arena_bytes=args.arena_gb << 30))
    tune_s = time.perf_counter() - t0
    probs = tuned.apply(probs)
    ecfg = tuned.engine
    for p in probs[:8]:
        G.solve(p, box_cap=4)
    t0 = time.perf_counter()
    plain = [G.solve(p, box_cap=4) for p in probs]
    t_plain = time.perf_counter() - t0
    with G.Engine(max_slots=args.count, arena_bytes=args.arena_gb << 30, threads=ecfg.threads,
                  blocks_per_sm=ecfg.blocks_per_sm, cand_mode=ecfg.cand_mode) as eng:
        eng.solve_all(probs[:8], box_cap=4)
        t0 = time.perf_counter()
        res = eng.solve_all(probs, box_cap=4)
        t_b = time.perf_counter() - t0
    same = all((a.lb, a.ub, a.iterations, a.status) == (b.lb, b.ub, b.iterations, b.status)
               for a, b in zip(plain, res))
    boxes = sum(r.boxes_bounded for r in res)
    return {"metric": "boxes/s", "value": boxes / t_b, "unit": "boxes/s", "n_gpus": 1, "dtype": "f64",
            "config": {"workload": f"cfg4-batch{args.count} with the full autotuner", "boxes": boxes,
                       "certified": sum(r.certified for r in res)},
            "batched_wall_s": t_b, "plain_wall_s": t_plain, "speedup_vs_plain": t_plain / t_b,
            "identical_to_plain": same, "engine": ecfg.label(),
            "autotune": {"seconds": tune_s, "fanout": {f"{lo}-{hi}": list(v) for (lo, hi), v in tuned.fanout.items()},
                         "matches_table": all(tuned.fanout.get(c) == v for c, v in A.TUNED_FANOUT.items()),
                         "trials": tuned.trials}}


def run_list_pass(args):
    """The grid-wide list pass on large lists: the 50-variable Rastrigin script's
    loop (4^10 children per iteration, rastrigin50.py:844-1289) for a few
    iterations; the list grows by about 1 Mi entries per iteration.  The pass
    is timed with the engine's phase stamps (GPUGO_PHASE_STAMPS) and its
    algorithmic bytes are 16 B per entry read plus 16 B per entry written."""
    import numpy as np
    path = os.path.join(tempfile.mkdtemp(), "stamps")
    os.environ["GPUGO_PHASE_STAMPS"] = path
    import gpugo_gb300 as G
    from gpugo_gb300 import problems as P
    n = 50
    p = P.Problem(P.COSQUAD, n, np.tile([-5.5, 6.0], n), np.concatenate([np.ones(n), np.full(n, 10.0), np.ones(n)]),
                  wid=4, group=10, samples=10, stop_mode=P.STOP_WIDTH, width_tol=1e-4, ub_init=1e6,
                  max_iter=args.steps, pool_cap=1 << 26)
    with G.Engine(max_slots=1, arena_bytes=8 << 30, threads=args.threads, blocks_per_sm=args.blocks_per_sm) as eng:
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
                                                      "iterations": int(st.shape[0]), "threads": args.threads,
                                                      "blocks_per_sm": args.blocks_per_sm},
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


def run_cfg3_full(args):
    """Config 3 as stated: the n = 32 exp-sqrt composite split in 2 parts per
    coordinate, 2^32 children per iteration, streamed through the candidate
    queue in passes (2^20 children each) with the list capped at --pool-gb.
    Every first-level child contains the minimiser at the centre of the domain,
    so none can be ruled out: the 2^32 survivors of the first iteration need a
    64 GiB list per buffer.  Runs --steps iterations (1 or 2) and reports the
    boxes bounded per second and how the solve ended (GPUGO_ERR_POOL_OVERFLOW,
    -4, when the cap is reached)."""
    import gpugo_gb300 as G
    from gpugo_gb300 import problems as P
    p = P.config3()
    p.max_iter = max(1, args.steps)
    pool_bytes = args.pool_gb << 30
    p.pool_cap = pool_bytes // 32              # two buffers of (LB, key) entries
    need = G.instance_bytes(p)
    with G.Engine(max_slots=1, arena_bytes=need + (64 << 20), wait_timeout_s=120.0) as eng:
        st0 = eng.stats()
        t0 = time.perf_counter()
        eng.submit(p, box_cap=4)
        eng.run(0)
        (_, r), = eng.poll()
        wall = time.perf_counter() - t0
        st1 = eng.stats()
    dev_s = (st1["total_run_ms"] - st0["total_run_ms"]) * 1e-3
    return {"metric": "boxes/s", "value": r.boxes_bounded / dev_s, "unit": "boxes/s", "n_gpus": 1, "dtype": "f64",
            "config": {"workload": "cfg3-expsqrt32 as stated: (2, 32) split, 2^32 children per iteration, children "
                                   f"streamed in passes of 2^20, list capped at {args.pool_gb} GiB",
                       "pool_cap_entries": p.pool_cap, "arena_bytes": need, "max_iter": p.max_iter},
            "status": r.status, "status_text": G._lib.ERRORS.get(r.status, "ok") if r.status < 0 else "solve state",
            "iterations": r.iterations, "boxes_bounded": r.boxes_bounded, "samples_evaluated": r.samples_evaluated,
            "pool_size": r.pool_size, "device_s": dev_s, "wall_s": wall, "ub": r.ub, "lb": r.lb,
            "kernel_launches": st1["kernel_launches"] - st0["kernel_launches"]}


def run_codelist(args):
    """The reference's seven benchmarks without a built-in family, as code
    lists (n = 8, split 3^8, UB-LB <= 1e-6), plus config 2 restated as a code
    list next to its built-in kernel; the CPU oracle solves each once."""
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
    ap.add_argument("--workload", default="batch",
                    choices=["batch", "cfg1", "cfg2", "cfg3", "cfg3-full", "cfg4-tune", "listpass", "codelist"],
                    help="batch is the benchmark line; the others print their own records")
    ap.add_argument("--count", type=int, default=1024, help="instances of the batch")
    ap.add_argument("--serve-count", type=int, default=4096, help="requests of the serving record (0: none)")
    ap.add_argument("--rate", type=float, default=20000.0)
    ap.add_argument("--slice", type=int, default=6, help="serving: iterations per run between admissions")
    ap.add_argument("--serve-order", default="shape", choices=["arrival", "shape"],
                    help="serving: waiting requests take free slots in arrival order or grouped by (family, n)")
    ap.add_argument("--arena-gb", type=int, default=80)
    ap.add_argument("--pool-gb", type=int, default=64, help="cfg3-full: list cap (two buffers)")
    ap.add_argument("--threads", type=int, default=256, help="listpass: threads per block (256 or 512)")
    ap.add_argument("--blocks-per-sm", type=int, default=2,
                    help="listpass: blocks per SM (two of 256 threads: six 32 KB tiles in flight per SM; 0: the "
                         "engine's choice for one instance, one block per SM)")
    ap.add_argument("--cpu-instances", type=int, default=64, help="batch instances the CPU baseline solves")
    ap.add_argument("--no-plain", dest="plain", action="store_false",
                    help="skip the plain one-instance-per-launch comparison")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip tuning the engine configuration (block size, candidates per warp)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    check_gpus(args.gpus)
    ws, rank, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args)
        if out is not None:
            print(json.dumps(out))
        return
    if args.workload != "batch":
        fn = {"cfg1": run_single, "cfg2": run_chained8, "cfg3": run_single, "cfg3-full": run_cfg3_full,
              "cfg4-tune": run_batched,
              "listpass": run_list_pass, "codelist": run_codelist}[args.workload]
        print(json.dumps(fn(args)))
        return
    dist = init_dist("nccl")
    out = run_batch(args, dist)
    if rank == 0:
        if args.cpu_instances > 0:
            out["cpu_baseline"] = run_cpu_baseline(batch_problems(args.count), args.cpu_instances)
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
