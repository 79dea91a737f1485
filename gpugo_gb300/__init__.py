"""gpugo_gb300 -- interval branch-and-bound global optimisation on GB300.

The per-problem call of the reference (one GPUGO script: objective, box domain
and stopping rule in; enclosure of the global minimum and surviving boxes out,
GPUGO_1.1/1-Ackley/ackley50.py:950-1396) is :func:`solve`.  :func:`eval_children`
is one sampling + ruleOutGPU pass (ackley50.py:602-766) over chosen children,
and :class:`Engine` runs many solves in one persistent kernel (batching and
serving).  All compute runs in libgpugo.so (hand-written CUDA for sm_103a);
Python only marshals arguments.  Objectives outside the four built-in families
are written with :mod:`gpugo_gb300.codelist` (family ``CODELIST``); the
reference's other benchmarks are in :mod:`gpugo_gb300.objectives`.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import CERTIFIED, FINISHED, ITER_LIMIT, GpugoError
from .problems import (CHAINED, CODELIST, COSQUAD, EXPSQRT, PRODCOS, STOP_GAP, STOP_WIDTH, Problem, config1,
                       config2, config3, config4, config5, instance)

__all__ = ["solve", "eval_children", "Engine", "SolveResult", "Problem", "GpugoError", "instance", "config1",
           "config2", "config3", "config4", "config5", "COSQUAD", "CHAINED", "EXPSQRT", "PRODCOS", "CODELIST",
           "STOP_GAP", "STOP_WIDTH", "CERTIFIED", "FINISHED", "ITER_LIMIT", "device_info", "combine",
           "checkpoint_ok"]

_dp = ctypes.POINTER(ctypes.c_double)
_SPEC = np.dtype(_lib.Spec)      # gpugo_spec as a NumPy record (a batch of them is one array)
_DONE = np.dtype(_lib.Done)      # gpugo_done as a NumPy record


def _f64(a) -> np.ndarray:
    """``a`` as a contiguous 1-D float64 array (itself when it already is one)."""
    if isinstance(a, np.ndarray) and a.dtype == np.float64 and a.ndim == 1 and a.flags.c_contiguous:
        return a
    return np.ascontiguousarray(a, dtype=np.float64).ravel()


def _spec(p: Problem):
    """The C ABI's gpugo_spec for ``p`` and the arrays it points into (keep them
    alive for the call).  Array addresses are taken from the array interface:
    a batch of a thousand problems is marshalled in a few milliseconds."""
    dom = _f64(p.domain)
    coef = _f64(p.coef)
    n = int(p.n)
    if dom.size != 2 * n:      # the library reads 2n bounds through a plain pointer
        raise ValueError(f"domain holds {dom.size} bounds, the problem needs 2n = {2 * n}")
    s = _lib.Spec(int(p.family), n, int(p.wid), int(p.group), int(p.samples), int(p.stop_mode),
                  float(p.width_tol), float(p.gap_tol), float(p.ub_init),
                  dom.__array_interface__["data"][0], coef.__array_interface__["data"][0], coef.size,
                  int(p.max_iter or 0), int(p.pool_cap or 0), int(p.parent_cap or 0))
    return s, (dom, coef)


@dataclass
class SolveResult:
    """Outcome of one solve: the reference prints ``[lb, ub]``, the output
    regions, the elapsed time and the iteration count (ackley50.py:1384-1395)."""
    lb: float
    ub: float
    status: int
    iterations: int
    boxes_bounded: int
    samples_evaluated: int
    pool_size: int
    n_boxes: int
    boxes: np.ndarray            # [k, n, 2]
    box_lbs: np.ndarray
    xhat: np.ndarray | None      # sample point whose upper bound is ub
    device_ms: float = 0.0
    trace: dict = field(default_factory=dict)

    @property
    def certified(self) -> bool:
        return self.status == CERTIFIED

    @property
    def gap(self) -> float:
        return self.ub - self.lb

    def record(self, tag: str = "") -> dict:
        """One structured log record of the solve (what the reference prints per
        script: enclosure, iterations, time; plus the work counts), JSON-ready;
        the survivors per iteration come from the trace when one was kept."""
        out = {"tag": tag, "lb": self.lb, "ub": self.ub, "gap": self.gap, "status": self.status,
               "certified": self.certified, "iterations": self.iterations, "boxes_bounded": self.boxes_bounded,
               "samples_evaluated": self.samples_evaluated, "pool_size": self.pool_size, "n_boxes": self.n_boxes,
               "device_ms": self.device_ms}
        if self.trace:
            out["survivors"] = [int(v) for v in self.trace["n_surv"]]
            out["list_sizes"] = [int(v) for v in self.trace["pool"]]
        return out


def _alloc_out(p: Problem, cap: int, trace_cap: int):
    boxes = np.zeros((max(cap, 1), 2 * p.n))
    lbs = np.zeros(max(cap, 1))
    xhat = np.zeros(p.n)
    tr = arrs = None
    if trace_cap > 0:
        arrs = (np.zeros(trace_cap), np.zeros(trace_cap, np.int64), np.zeros(trace_cap, np.int64),
                np.zeros(trace_cap, np.int64))
        i64 = ctypes.POINTER(ctypes.c_int64)
        tr = _lib.Trace(trace_cap, arrs[0].ctypes.data_as(_dp), arrs[1].ctypes.data_as(i64),
                        arrs[2].ctypes.data_as(i64), arrs[3].ctypes.data_as(i64))
    return boxes, lbs, xhat, tr, arrs


def _result(p: Problem, r, boxes, lbs, xhat, arrs) -> SolveResult:
    k = int(r.n_out)
    trace = {}
    if arrs is not None:
        m = min(int(r.iterations), arrs[0].size)
        trace = {"ub": arrs[0][:m].copy(), "n_surv": arrs[1][:m].copy(), "pool": arrs[2][:m].copy(),
                 "sel": arrs[3][:m].copy()}
    return SolveResult(float(r.lb), float(r.ub), int(r.status), int(r.iterations), int(r.boxes_bounded),
                       int(r.samples_evaluated), int(r.pool_size), int(r.n_boxes),
                       boxes[:k].reshape(k, p.n, 2).copy(), lbs[:k].copy(),
                       xhat.copy() if r.has_xhat else None, float(r.device_ms), trace)


def solve(p: Problem, box_cap: int = 1024, trace_cap: int = 0) -> SolveResult:
    """Solve one problem on the GPU (libgpugo.so ``gpugo_solve``)."""
    L = _lib.load()
    s, keep = _spec(p)
    boxes, lbs, xhat, tr, arrs = _alloc_out(p, box_cap, trace_cap)
    r = _lib.Result()
    rc = L.gpugo_solve(ctypes.byref(s), ctypes.byref(r), boxes.ctypes.data_as(_dp), lbs.ctypes.data_as(_dp),
                       box_cap, xhat.ctypes.data_as(_dp), ctypes.byref(tr) if tr is not None else None)
    _lib.check(rc, "gpugo_solve")
    return _result(p, r, boxes, lbs, xhat, arrs)


def eval_children(p: Problem, parent_box: np.ndarray, cyc: int, codes: np.ndarray, ub: float):
    """Per child: lower bound, smallest sampled upper bound, ruleOutGPU flag."""
    L = _lib.load()
    s, keep = _spec(p)
    pb = np.ascontiguousarray(parent_box, dtype=np.float64).ravel()
    if pb.size != 2 * int(p.n):
        raise ValueError(f"parent box holds {pb.size} bounds, the problem needs 2n = {2 * int(p.n)}")
    codes = np.ascontiguousarray(codes, dtype=np.uint64).ravel()
    m = codes.size
    lb = np.empty(m)
    samp = np.empty(m)
    flag = np.empty(m, dtype=np.int32)
    rc = L.gpugo_eval_children(ctypes.byref(s), pb.ctypes.data_as(_dp), int(cyc),
                               codes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), m, float(ub),
                               lb.ctypes.data_as(_dp), samp.ctypes.data_as(_dp),
                               flag.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    _lib.check(rc, "gpugo_eval_children")
    return lb, samp, flag


def checkpoint_ok(data: bytes) -> bool:
    """Whether ``Engine.restore`` would accept a checkpoint (``gpugo_checkpoint_check``:
    the problem, the state and every index the lists hold), checked on the host."""
    buf = ctypes.create_string_buffer(bytes(data), len(data))
    return _lib.load().gpugo_checkpoint_check(buf, len(data)) == 0


def combine(boxes: np.ndarray, tol: float = 1e-3) -> np.ndarray:
    """Merge result boxes ([k, n, 2], in emission order) into connected roots on
    the GPU (``gpugo_combine``; the reference's combine / connectivity,
    rosenbrock50.py:926-1049, with its combineTolerance 1e-3 as the default)."""
    L = _lib.load()
    b = np.ascontiguousarray(boxes, dtype=np.float64)
    k, n = int(b.shape[0]), int(b.shape[1])
    out = np.empty((max(k, 1), n, 2))
    nr = ctypes.c_int64()
    _lib.check(L.gpugo_combine(b.ctypes.data_as(_dp), k, n, float(tol), out.ctypes.data_as(_dp), k,
                               ctypes.byref(nr)), "gpugo_combine")
    return out[:nr.value].copy()


def device_info() -> tuple[int, int]:
    L = _lib.load()
    sm = ctypes.c_int32()
    nsm = ctypes.c_int32()
    _lib.check(L.gpugo_device_info(ctypes.byref(sm), ctypes.byref(nsm)), "gpugo_device_info")
    return sm.value, nsm.value


def instance_bytes(p: Problem) -> int:
    L = _lib.load()
    s, keep = _spec(p)
    out = ctypes.c_int64()
    _lib.check(L.gpugo_instance_bytes(ctypes.byref(s), ctypes.byref(out)), "gpugo_instance_bytes")
    return out.value


class Engine:
    """Many solves resident on one GPU, advanced together by one persistent kernel.

    ``submit`` admits a problem when a slot and enough pool memory are free
    (``None`` otherwise), ``run`` advances every resident solve, ``poll`` returns
    the finished ones and frees their memory.
    """

    def __init__(self, max_slots: int = 1024, arena_bytes: int = 8 << 30, wait_timeout_s: float = 60.0,
                 blocks_per_sm: int = 0, cand_mode: int = _lib.CAND_AUTO, threads: int = 256, chunk_children: int = 0):
        self._L = _lib.load()
        cfg = _lib.EngineCfg(int(max_slots), int(threads), int(arena_bytes), float(wait_timeout_s),
                             int(blocks_per_sm), int(cand_mode), int(chunk_children))
        h = ctypes.c_void_p()
        _lib.check(self._L.gpugo_engine_create(ctypes.byref(cfg), ctypes.byref(h)), "gpugo_engine_create")
        self._h = h
        self._pending: dict[int, tuple] = {}
        self.max_slots = max_slots

    def close(self):
        if self._h:
            self._L.gpugo_engine_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, p: Problem, box_cap: int = 16, trace_cap: int = 0) -> int | None:
        s, keep = _spec(p)
        boxes, lbs, xhat, tr, arrs = _alloc_out(p, box_cap, trace_cap)
        t = ctypes.c_int64()
        rc = self._L.gpugo_submit(self._h, ctypes.byref(s), boxes.__array_interface__["data"][0],
                                  lbs.__array_interface__["data"][0], box_cap, xhat.__array_interface__["data"][0],
                                  ctypes.byref(tr) if tr is not None else None, ctypes.byref(t))
        if rc == _lib.ERR_BUSY:
            return None
        _lib.check(rc, "gpugo_submit")
        self._pending[t.value] = (p, boxes, lbs, xhat, arrs, tr, keep)
        return t.value

    def submit_many(self, problems: list[Problem], box_cap: int = 16) -> list[int]:
        """Admit ``problems`` in order with one ``gpugo_submit_batch`` call, as many
        as fit: returns the tickets of the admitted prefix (shorter than
        ``problems`` when the engine filled up).  Their results come from ``poll``
        as for ``submit``; the descriptions are gathered column by column and the
        output buffers are three arrays shared by the batch.  A description the
        library refuses raises ``GpugoError`` whose ``admitted`` lists the tickets
        of the problems before it (admitted all the same); a domain of the wrong
        size raises ``ValueError`` before anything is admitted."""
        m = len(problems)
        if m == 0:
            return []
        ns = np.fromiter((p.n for p in problems), np.int64, m)
        doms = [_f64(p.domain) for p in problems]
        coefs = [_f64(p.coef) for p in problems]
        dsz = np.fromiter((d.size for d in doms), np.int64, m)
        bad = np.flatnonzero(dsz != 2 * ns)
        if bad.size:       # the library reads 2n bounds through a plain pointer
            i = int(bad[0])
            raise ValueError(f"problem {i}: domain holds {dsz[i]} bounds, the problem needs 2n = {2 * ns[i]}")
        csz = np.fromiter((c.size for c in coefs), np.int64, m)
        dom = np.concatenate(doms)
        coef = np.concatenate(coefs) if csz.sum() else np.zeros(1)
        specs = np.zeros(m, _SPEC)
        for name in ("family", "wid", "group", "samples", "stop_mode", "width_tol", "gap_tol", "ub_init"):
            specs[name] = [getattr(p, name) for p in problems]
        for name in ("max_iter", "pool_cap", "parent_cap"):
            specs[name] = [getattr(p, name) or 0 for p in problems]
        specs["n"] = ns
        specs["ncoef"] = csz
        specs["domain"] = dom.ctypes.data + 8 * (np.cumsum(dsz) - dsz)
        specs["coef"] = coef.ctypes.data + 8 * (np.cumsum(csz) - csz)
        at = np.cumsum(ns) - ns                      # N_i: coordinates before problem i
        cap = int(box_cap)
        boxes = np.zeros(2 * cap * int(ns.sum()))
        lbs = np.zeros(cap * m)
        xhat = np.zeros(int(ns.sum()))
        tickets = np.zeros(m, np.int64)
        done = ctypes.c_int64()
        rc = self._L.gpugo_submit_batch(self._h, specs.ctypes.data, m, boxes.ctypes.data, lbs.ctypes.data, cap,
                                        xhat.ctypes.data, tickets.ctypes.data, ctypes.byref(done))
        k = done.value
        # admitted problems are registered before an error is raised; their parts
        # of the shared buffers are cut out when their results come (poll)
        out = (boxes, lbs, xhat, cap)
        self._pending.update(zip(tickets[:k].tolist(),
                                 ((q, None, None, None, None, None, (out, i, a))
                                  for i, (q, a) in enumerate(zip(problems[:k], at[:k].tolist())))))
        if rc < 0 and rc != _lib.ERR_BUSY:
            err = GpugoError(rc, f"gpugo_submit_batch (problem {k})")
            err.admitted = tickets[:k].tolist()
            raise err
        return tickets[:k].tolist()

    def checkpoint(self, ticket: int) -> bytes:
        """Serialise a resident solve (between runs): problem, state, parent table,
        list, emitted boxes and trace."""
        size = ctypes.c_int64()
        _lib.check(self._L.gpugo_checkpoint(self._h, int(ticket), None, 0, ctypes.byref(size)), "gpugo_checkpoint")
        buf = ctypes.create_string_buffer(size.value)
        _lib.check(self._L.gpugo_checkpoint(self._h, int(ticket), buf, size.value, ctypes.byref(size)),
                   "gpugo_checkpoint")
        return buf.raw[:size.value]

    def restore(self, p: Problem, data: bytes, box_cap: int = 16, trace_cap: int = 0) -> int | None:
        """Admit a checkpointed solve of problem ``p``; it continues where the
        checkpoint was taken.  ``None`` when no slot or memory is free."""
        boxes, lbs, xhat, tr, arrs = _alloc_out(p, box_cap, trace_cap)
        t = ctypes.c_int64()
        buf = ctypes.create_string_buffer(bytes(data), len(data))
        rc = self._L.gpugo_restore(self._h, buf, len(data), boxes.ctypes.data_as(_dp), lbs.ctypes.data_as(_dp),
                                   box_cap, xhat.ctypes.data_as(_dp), ctypes.byref(tr) if tr is not None else None,
                                   ctypes.byref(t))
        if rc == _lib.ERR_BUSY:
            return None
        _lib.check(rc, "gpugo_restore")
        self._pending[t.value] = (p, boxes, lbs, xhat, arrs, tr, None)
        return t.value

    def run(self, max_iters: int = 0) -> int:
        active = ctypes.c_int32()
        _lib.check(self._L.gpugo_run(self._h, int(max_iters), ctypes.byref(active)), "gpugo_run")
        return active.value

    def poll(self, max_done: int = 4096) -> list[tuple[int, SolveResult]]:
        arr = (_lib.Done * max_done)()
        nd = ctypes.c_int32()
        _lib.check(self._L.gpugo_poll(self._h, arr, max_done, ctypes.byref(nd)), "gpugo_poll")
        out = []
        m = nd.value
        if m == 0:
            return out
        # the records read column by column (a batch returns a thousand at once);
        # boxes, LBs and points are views of the buffers allocated at admission
        rec = np.frombuffer(arr, _DONE, m)
        res = rec["result"]
        cols = [res[f].tolist() for f in ("lb", "ub", "status", "iterations", "boxes_bounded",
                                          "samples_evaluated", "pool_size", "n_boxes", "n_out", "has_xhat",
                                          "device_ms")]
        rows = zip(rec["ticket"].tolist(), *cols)
        for i, (t, lb, ub, status, iters, bb, se, ps, nb, k, hx, dms) in enumerate(rows):
            p, boxes, lbs, xhat, arrs, tr, keep = self._pending.pop(t)
            n = p.n
            if boxes is None:
                # a batch admission (submit_many): problem j's parts of the shared buffers
                (bx, bl, bh, cap), j, at = keep
                out.append((t, SolveResult(lb, ub, status, iters, bb, se, ps, nb,
                                           bx[2 * cap * at:2 * cap * at + 2 * n * k].reshape(k, n, 2),
                                           bl[cap * j:cap * j + k], bh[at:at + n] if hx else None, dms)))
                continue
            if arrs is not None:
                out.append((t, _result(p, arr[i].result, boxes, lbs, xhat, arrs)))
                continue
            out.append((t, SolveResult(lb, ub, status, iters, bb, se, ps, nb, boxes[:k].reshape(k, n, 2),
                                       lbs[:k], xhat if hx else None, dms)))
        return out

    def stats(self) -> dict:
        """Engine counters: device time of the runs, kernel launches, iterations, copies."""
        st = _lib.Stats()
        _lib.check(self._L.gpugo_engine_stats(self._h, ctypes.byref(st)), "gpugo_engine_stats")
        return {"last_run_ms": st.last_run_ms, "total_run_ms": st.total_run_ms,
                "kernel_launches": st.kernel_launches, "iterations": st.iterations,
                "h2d_bytes": st.h2d_bytes, "d2h_bytes": st.d2h_bytes}

    def free_bytes(self) -> int:
        out = ctypes.c_int64()
        _lib.check(self._L.gpugo_engine_free_bytes(self._h, ctypes.byref(out)), "gpugo_engine_free_bytes")
        return out.value

    def solve_all(self, problems: list[Problem], iters_per_run: int = 0, box_cap: int = 16,
                  group_by_shape: bool = True):
        """Admit as many problems as fit, run, collect, refill; returns results in input order.
        ``group_by_shape`` admits them ordered by (family, n): slots, and so the
        kernel's work lists, then hold neighbours of equal cost side by side."""
        results: list[SolveResult | None] = [None] * len(problems)
        tickets: dict[int, int] = {}
        order = list(range(len(problems)))
        if group_by_shape:
            order.sort(key=lambda k: (problems[k].family, problems[k].n))
        nxt = 0
        while nxt < len(problems) or tickets:
            if nxt < len(problems):
                for t in self.submit_many([problems[k] for k in order[nxt:]], box_cap=box_cap):
                    tickets[t] = order[nxt]
                    nxt += 1
            if not tickets:
                raise GpugoError(-7, f"problem {order[nxt]} does not fit an empty engine")
            self.run(iters_per_run)
            for t, r in self.poll():
                results[tickets.pop(t)] = r
        return results
