"""Continuous-batching request loop over one GPU.

Solve requests arrive over time (a Poisson stream in the benchmark).  A request
is admitted into the resident engine as soon as a slot and enough box-pool memory
are free (``Engine.submit`` refuses otherwise); every resident solve keeps its
list and UB on the device and advances inside the same persistent kernel; the
kernel returns every ``slice_iters`` iterations so that finished solves are
collected and waiting requests join the running batch.  A request the library
refuses (an invalid description) or one too large for the empty engine is
answered with its error (``RequestRecord.error``) and the stream goes on; a
device or CUDA failure ends the run.

The reference has no serving mode: each script solves one problem
(GPUGO_1.1/1-Ackley/ackley50.py:950-1396).
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import Engine, SolveResult, _lib
from .problems import Problem


@dataclass
class RequestRecord:
    index: int
    arrival: float                 # seconds after the start of the run
    admitted: float = -1.0
    finished: float = -1.0
    result: SolveResult | None = None
    error: str | None = None       # why the request was refused (then result is None)

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


@dataclass
class ServeReport:
    records: list[RequestRecord]
    wall_s: float
    device_s: float
    launches: int
    engine_iterations: int
    boxes: int = 0
    certified: int = 0
    rejected: int = 0
    p50_ms: float = 0.0
    p99_ms: float = 0.0
    extra: dict = field(default_factory=dict)

    def summary(self) -> dict:
        return {"requests": len(self.records), "certified": self.certified, "rejected": self.rejected,
                "wall_s": self.wall_s,
                "device_s": self.device_s, "boxes": self.boxes, "boxes_per_s": self.boxes / self.wall_s,
                "p50_ms": self.p50_ms, "p99_ms": self.p99_ms, "kernel_launches": self.launches,
                "engine_iterations": self.engine_iterations, **self.extra}


def serve(stream: list[tuple[float, Problem]], max_slots: int = 1024, arena_bytes: int = 80 << 30,
          slice_iters: int = 16, box_cap: int = 4, engine: Engine | None = None,
          clock=time.perf_counter, order: str = "arrival") -> ServeReport:
    """Run ``stream`` (pairs of arrival time in seconds and problem, sorted by
    arrival) through one engine; returns per-request latencies and results.
    ``order`` is how waiting requests take free slots: ``"arrival"`` first come
    first served, ``"shape"`` grouped by (family, n) and then by arrival, so that
    neighbouring slots (and so the kernel's work lists) hold solves of one shape."""
    if order not in ("arrival", "shape"):
        raise ValueError(f"order {order!r}")
    own = engine is None
    eng = engine or Engine(max_slots=max_slots, arena_bytes=arena_bytes)
    records = [RequestRecord(i, float(t)) for i, (t, _) in enumerate(stream)]
    pending: deque[int] = deque()
    nxt = 0
    tickets: dict[int, int] = {}
    st0 = eng.stats()
    t0 = clock()
    done = 0
    while done < len(records):
        now = clock() - t0
        arrived = False
        while nxt < len(records) and stream[nxt][0] <= now:
            pending.append(nxt)
            nxt += 1
            arrived = True
        if arrived and order == "shape" and len(pending) > 1:
            pending = deque(sorted(pending, key=lambda k: (stream[k][1].family, stream[k][1].n, k)))
        # admit in arrival order while slots and pool memory last; a request the
        # library refuses (a bad description) or that cannot fit even an empty
        # engine is answered with its error and the stream goes on
        while pending:
            i = pending[0]
            try:
                t = eng.submit(stream[i][1], box_cap=box_cap)
            except _lib.GpugoError as e:
                if e.code != _lib.ERR_INVALID:      # a device or CUDA failure ends the run
                    raise
                t, records[i].error = None, str(e)
            except ValueError as e:                 # arrays of the wrong size
                t, records[i].error = None, str(e)
            if t is None and records[i].error is None and not tickets:
                records[i].error = "does not fit an empty engine"
            if records[i].error is not None:
                pending.popleft()
                records[i].finished = clock() - t0
                done += 1
                continue
            if t is None:
                break
            pending.popleft()
            tickets[t] = i
            records[i].admitted = clock() - t0
        if not tickets:
            # idle until the next arrival
            if nxt < len(records):
                wait = stream[nxt][0] - (clock() - t0)
                if wait > 0:
                    time.sleep(min(wait, 0.001))
            continue
        eng.run(slice_iters)
        fin = clock() - t0
        for t, r in eng.poll():
            i = tickets.pop(t)
            records[i].finished = fin
            records[i].result = r
            done += 1
    wall = clock() - t0
    st1 = eng.stats()
    if own:
        eng.close()
    served = [r for r in records if r.result is not None]
    lat = np.array([r.latency for r in served]) * 1e3
    rep = ServeReport(records, wall, (st1["total_run_ms"] - st0["total_run_ms"]) * 1e-3,
                      int(st1["kernel_launches"] - st0["kernel_launches"]),
                      int(st1["iterations"] - st0["iterations"]))
    rep.boxes = sum(r.result.boxes_bounded for r in served)
    rep.certified = sum(r.result.certified for r in served)
    rep.rejected = len(records) - len(served)
    if served:
        rep.p50_ms = float(np.percentile(lat, 50))
        rep.p99_ms = float(np.percentile(lat, 99))
    return rep


# ---------------------------------------------------------------------------
# several GPUs: one process and one engine per GPU, arrivals dealt round-robin
# ---------------------------------------------------------------------------
def partition_stream(stream: list[tuple[float, Problem]], rank: int, world: int) -> list[tuple[float, Problem]]:
    """The requests rank ``rank`` of ``world`` serves: every world-th arrival,
    starting at the rank's index, with the arrival times kept.  Requests are
    independent, so no data crosses between ranks while they are served."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    return stream[rank::world]


def latency_record(rep: ServeReport) -> dict:
    """What one rank contributes to the merged report: its served latencies (ms),
    counts and wall time (plain numbers, so that it can cross process boundaries)."""
    served = [r for r in rep.records if r.result is not None]
    return {"latencies_ms": [r.latency * 1e3 for r in served], "boxes": rep.boxes, "certified": rep.certified,
            "rejected": rep.rejected, "requests": len(rep.records), "wall_s": rep.wall_s, "device_s": rep.device_s,
            "launches": rep.launches}


def merge_records(recs: list[dict]) -> dict:
    """Merged serving figures over ranks: p50/p99 over every served request's
    latency, boxes and certified solves summed, boxes/s over the slowest rank's
    wall time (the job ends when the last rank does)."""
    lat = np.array([x for r in recs for x in r["latencies_ms"]], dtype=np.float64)
    wall = max(r["wall_s"] for r in recs)
    boxes = sum(r["boxes"] for r in recs)
    return {"ranks": len(recs), "requests": sum(r["requests"] for r in recs),
            "certified": sum(r["certified"] for r in recs), "rejected": sum(r["rejected"] for r in recs),
            "wall_s": wall, "device_s_max": max(r["device_s"] for r in recs), "boxes": boxes,
            "boxes_per_s": boxes / wall if wall > 0 else 0.0,
            "p50_ms": float(np.percentile(lat, 50)) if lat.size else 0.0,
            "p99_ms": float(np.percentile(lat, 99)) if lat.size else 0.0,
            "kernel_launches": sum(r["launches"] for r in recs)}


def serve_sharded(stream: list[tuple[float, Problem]], dist=None, **kw) -> dict | None:
    """Serve ``stream`` across the ranks of ``dist`` (torch.distributed, already
    initialised; None for one process): each rank serves its round-robin share
    on its own GPU, then rank 0 gathers the per-rank records and returns the
    merged figures (other ranks return None).  The only collective is that
    gather, after the stream has been served."""
    world = dist.get_world_size() if dist is not None else 1
    rank = dist.get_rank() if dist is not None else 0
    rep = serve(partition_stream(stream, rank, world), **kw)
    rec = latency_record(rep)
    if dist is None:
        return merge_records([rec])
    out = [None] * world if rank == 0 else None
    dist.gather_object(rec, out, dst=0)
    return merge_records(out) if rank == 0 else None
