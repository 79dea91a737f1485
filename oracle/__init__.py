"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is the parity checker for the GPU path: only the tests, the smoke
check and the CPU-baseline leg of ``bench.py`` import this package.  The product
(``gpugo_gb300``) never imports it and has no CPU fallback.

``solve`` mirrors the reference's host B&B loop (GPUGO_1.1/1-Ackley/ackley50.py:950-1396)
and ``eval_children`` one ``sampling`` + ``ruleOutGPU`` pass (ackley50.py:602-766).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgpugo_oracle.so")
# another build of the same source (e.g. `make -C oracle asan`), used as is
_LIB_OVERRIDE = os.environ.get("GPUGO_ORACLE_LIB")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, no GPU needed)."""
    if _LIB_OVERRIDE:
        return _LIB_OVERRIDE
    src = os.path.join(_HERE, "gpugo_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Spec(ctypes.Structure):
    _fields_ = [
        ("family", ctypes.c_int32), ("n", ctypes.c_int32), ("wid", ctypes.c_int32),
        ("group", ctypes.c_int32), ("samples", ctypes.c_int32), ("stop_mode", ctypes.c_int32),
        ("width_tol", ctypes.c_double), ("gap_tol", ctypes.c_double), ("ub_init", ctypes.c_double),
        ("domain", ctypes.POINTER(ctypes.c_double)), ("coef", ctypes.POINTER(ctypes.c_double)),
        ("ncoef", ctypes.c_int64), ("max_iter", ctypes.c_int64), ("pool_cap", ctypes.c_int64),
        ("parent_cap", ctypes.c_int64),
    ]


class _Result(ctypes.Structure):
    _fields_ = [
        ("lb", ctypes.c_double), ("ub", ctypes.c_double), ("n_boxes", ctypes.c_int64),
        ("iterations", ctypes.c_int64), ("boxes_bounded", ctypes.c_int64), ("pool_size", ctypes.c_int64),
        ("status", ctypes.c_int32), ("n_out", ctypes.c_int32), ("samples_evaluated", ctypes.c_int64),
    ]


class _Trace(ctypes.Structure):
    _fields_ = [
        ("cap", ctypes.c_int64), ("ub", ctypes.POINTER(ctypes.c_double)),
        ("n_surv", ctypes.POINTER(ctypes.c_int64)), ("pool", ctypes.POINTER(ctypes.c_int64)),
        ("sel", ctypes.POINTER(ctypes.c_int64)),
    ]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_OVERRIDE or _LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.oc_ia_op.argtypes = [ctypes.c_int, ctypes.c_long, dp, dp, dp]
        L.oc_round_op.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, dp, dp, dp]
        L.oc_point_fn.argtypes = [ctypes.c_int, ctypes.c_long, dp, dp]
        L.oc_child_box.argtypes = [ctypes.POINTER(_Spec), dp, ctypes.c_int, ctypes.c_uint64, dp]
        L.oc_eval_children.argtypes = [ctypes.POINTER(_Spec), dp, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_uint64), ctypes.c_long, ctypes.c_double,
                                       dp, dp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
        L.oc_solve.argtypes = [ctypes.POINTER(_Spec), ctypes.c_int, ctypes.POINTER(_Result), dp, dp,
                               ctypes.c_int64, ctypes.POINTER(_Trace)]
        L.oc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


IA_OPS = {"add": 0, "minus": 1, "mul": 2, "div": 3, "sqr": 4, "sqrt": 5, "times": 6, "plus": 7,
          "sin": 8, "cos": 9, "exp": 10}


def ia_op(op: str, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    """Apply one interval op to m intervals (arrays of shape [m, 2])."""
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 2)
    out = np.empty_like(a)
    bp = None
    if b is not None:
        b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1, 2)
        bp = _dp(b)
    lib().oc_ia_op(IA_OPS[op], a.shape[0], _dp(a), bp, _dp(out))
    return out


def round_op(op: str, direction: str, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    ops = {"add": 0, "mul": 1, "div": 2, "sqrt": 3}
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    b = np.ascontiguousarray(b if b is not None else np.zeros_like(a), dtype=np.float64).ravel()
    out = np.empty_like(a)
    lib().oc_round_op(ops[op], 0 if direction == "down" else 1, a.size, _dp(a), _dp(b), _dp(out))
    return out


def point_fn(fn: str, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    out = np.empty_like(x)
    lib().oc_point_fn({"exp": 0, "sin": 1, "cos": 2}[fn], x.size, _dp(x), _dp(out))
    return out


def _spec(p):
    dom = np.ascontiguousarray(p.domain, dtype=np.float64).ravel()
    coef = np.ascontiguousarray(p.coef, dtype=np.float64).ravel()
    s = _Spec(int(p.family), int(p.n), int(p.wid), int(p.group), int(p.samples), int(p.stop_mode),
              float(p.width_tol), float(p.gap_tol), float(p.ub_init), _dp(dom), _dp(coef), coef.size,
              int(getattr(p, "max_iter", 0) or 0), int(getattr(p, "pool_cap", 0) or 0),
              int(getattr(p, "parent_cap", 0) or 0))
    return s, (dom, coef)


def child_box(p, pbox: np.ndarray, cyc: int, code: int) -> np.ndarray:
    s, keep = _spec(p)
    pb = np.ascontiguousarray(pbox, dtype=np.float64).ravel()
    out = np.empty(2 * p.n)
    rc = lib().oc_child_box(ctypes.byref(s), _dp(pb), int(cyc), int(code), _dp(out))
    if rc:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return out


def eval_children(p, pbox: np.ndarray, cyc: int, codes: np.ndarray, ub: float):
    """Per child: (lb, smallest sampled upper bound, ruleOut flag, derivative flag)."""
    s, keep = _spec(p)
    pb = np.ascontiguousarray(pbox, dtype=np.float64).ravel()
    codes = np.ascontiguousarray(codes, dtype=np.uint64).ravel()
    m = codes.size
    lb = np.empty(m); samp = np.empty(m)
    flag = np.empty(m, dtype=np.int32); dflag = np.empty(m, dtype=np.int32)
    rc = lib().oc_eval_children(ctypes.byref(s), _dp(pb), int(cyc),
                                codes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), m, float(ub),
                                _dp(lb), _dp(samp), flag.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                dflag.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    if rc:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return lb, samp, flag, dflag


@dataclass
class OracleResult:
    lb: float
    ub: float
    n_boxes: int
    iterations: int
    boxes_bounded: int
    pool_size: int
    status: int
    samples_evaluated: int
    boxes: np.ndarray
    box_lbs: np.ndarray
    trace: dict


def solve(p, box_cap: int = 4096, trace_cap: int = 0, skip_samples: bool = True) -> OracleResult:
    """Run the reference B&B loop on the CPU.  ``skip_samples`` leaves out the
    sample evaluation of children whose LB already exceeds the running UB;
    the UB sequence and every decision are unchanged by it."""
    s, keep = _spec(p)
    res = _Result()
    boxes = np.zeros((max(box_cap, 1), 2 * p.n))
    lbs = np.zeros(max(box_cap, 1))
    tr = None
    arrs = None
    if trace_cap > 0:
        arrs = (np.zeros(trace_cap), np.zeros(trace_cap, np.int64), np.zeros(trace_cap, np.int64),
                np.zeros(trace_cap, np.int64))
        tr = _Trace(trace_cap, _dp(arrs[0]), arrs[1].ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                    arrs[2].ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                    arrs[3].ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    lib().oc_solve(ctypes.byref(s), 1 if skip_samples else 0, ctypes.byref(res), _dp(boxes), _dp(lbs),
                   box_cap, ctypes.byref(tr) if tr is not None else None)
    n_out = res.n_out
    trace = {}
    if arrs is not None:
        k = min(res.iterations, trace_cap)
        trace = {"ub": arrs[0][:k].copy(), "n_surv": arrs[1][:k].copy(), "pool": arrs[2][:k].copy(),
                 "sel": arrs[3][:k].copy()}
    return OracleResult(res.lb, res.ub, res.n_boxes, res.iterations, res.boxes_bounded, res.pool_size,
                        res.status, res.samples_evaluated, boxes[:n_out].copy(), lbs[:n_out].copy(), trace)


def combine(boxes: np.ndarray, tol: float) -> np.ndarray:
    """Result-box merging in order (rosenbrock50.py:926-1049); boxes [k, n, 2]."""
    b = np.ascontiguousarray(boxes, dtype=np.float64)
    k, n = b.shape[0], b.shape[1]
    out = np.empty_like(b) if k else np.empty((0, n, 2))
    L = lib()
    L.oc_combine.restype = ctypes.c_int64
    L.oc_combine.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int64, ctypes.c_int, ctypes.c_double,
                             ctypes.POINTER(ctypes.c_double), ctypes.c_int64]
    nr = L.oc_combine(_dp(b.reshape(-1)) if k else None, k, n, float(tol), _dp(out.reshape(-1)) if k else None, k)
    return out[:nr].copy()


def num_threads() -> int:
    return int(lib().oc_num_threads())
