"""ctypes binding of libgpugo.so (the C ABI in include/gpugo.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback for any call.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

GPUGO_OK = 0
ERRORS = {
    -1: "invalid problem or argument", -2: "CUDA runtime error", -3: "out of memory",
    -4: "box pool capacity exceeded", -5: "parent table capacity exceeded",
    -6: "a bounded device wait expired", -7: "no free slot or pool memory",
    -8: "unknown ticket", -9: "no CUDA device",
    -10: "request exceeds the fixed scratch of gpugo_eval_children_static",
}
CERTIFIED, FINISHED, ITER_LIMIT = 1, 2, 3
CAND_AUTO, CAND_WARP, CAND_LANE = 0, 1, 2
ERR_INVALID, ERR_BUSY = -1, -7

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


class Spec(ctypes.Structure):
    _fields_ = [
        ("family", ctypes.c_int32), ("n", ctypes.c_int32), ("wid", ctypes.c_int32),
        ("group", ctypes.c_int32), ("samples", ctypes.c_int32), ("stop_mode", ctypes.c_int32),
        ("width_tol", ctypes.c_double), ("gap_tol", ctypes.c_double), ("ub_init", ctypes.c_double),
        # const double* (addresses of float64 arrays; c_void_p takes them as integers)
        ("domain", ctypes.c_void_p), ("coef", ctypes.c_void_p), ("ncoef", ctypes.c_int64), ("max_iter", ctypes.c_int64),
        ("pool_cap", ctypes.c_int64), ("parent_cap", ctypes.c_int64),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("lb", ctypes.c_double), ("ub", ctypes.c_double), ("n_boxes", ctypes.c_int64),
        ("iterations", ctypes.c_int64), ("boxes_bounded", ctypes.c_int64), ("pool_size", ctypes.c_int64),
        ("status", ctypes.c_int32), ("n_out", ctypes.c_int32), ("samples_evaluated", ctypes.c_int64),
        ("has_xhat", ctypes.c_int32), ("reserved", ctypes.c_int32), ("device_ms", ctypes.c_double),
        ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64),
    ]


class Stats(ctypes.Structure):
    _fields_ = [("last_run_ms", ctypes.c_double), ("total_run_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("iterations", ctypes.c_int64),
                ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]


class Trace(ctypes.Structure):
    _fields_ = [("cap", ctypes.c_int64), ("ub", _dp), ("n_surv", _i64p), ("pool", _i64p), ("sel", _i64p)]


class EngineCfg(ctypes.Structure):
    _fields_ = [
        ("max_slots", ctypes.c_int32), ("threads", ctypes.c_int32), ("arena_bytes", ctypes.c_int64),
        ("wait_timeout_s", ctypes.c_double), ("blocks_per_sm", ctypes.c_int32), ("cand_mode", ctypes.c_int32),
        ("chunk_children", ctypes.c_int64),
    ]


class Done(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_int64), ("result", Result)]


# every symbol include/gpugo.h declares
EXPORTS = [
    "gpugo_solve", "gpugo_eval_children", "gpugo_engine_create", "gpugo_engine_destroy", "gpugo_submit",
    "gpugo_run", "gpugo_poll", "gpugo_engine_free_bytes", "gpugo_instance_bytes", "gpugo_strerror",
    "gpugo_device_info", "gpugo_engine_stats", "gpugo_fp64_peak", "gpugo_eval_children_static",
    "gpugo_combine", "gpugo_checkpoint", "gpugo_restore", "gpugo_checkpoint_check", "gpugo_submit_batch",
]

_lib = None


class GpugoError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {ERRORS.get(code, code)} ({code})" if what else f"{ERRORS.get(code, code)} ({code})")


def path() -> str:
    """The library loaded: the in-tree build, or another build of the same
    source named by GPUGO_LIB (e.g. the host-sanitizer build of
    ``build.build_host_asan``)."""
    return os.environ.get("GPUGO_LIB") or _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libgpugo.so; raises when it is missing (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path()
    if build_if_missing and not os.path.exists(p):
        _build.build()
    if not os.path.exists(p):
        raise ImportError(f"libgpugo.so is not built ({p}); run gpugo_gb300.build.build() or "
                          f"__graft_entry__.build() first")
    L = ctypes.CDLL(p)
    vp = ctypes.c_void_p
    L.gpugo_solve.argtypes = [ctypes.POINTER(Spec), ctypes.POINTER(Result), _dp, _dp, ctypes.c_int64, _dp,
                              ctypes.POINTER(Trace)]
    L.gpugo_eval_children.argtypes = [ctypes.POINTER(Spec), _dp, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64),
                                      ctypes.c_int64, ctypes.c_double, _dp, _dp, ctypes.POINTER(ctypes.c_int32)]
    L.gpugo_eval_children_static.argtypes = L.gpugo_eval_children.argtypes
    L.gpugo_engine_create.argtypes = [ctypes.POINTER(EngineCfg), ctypes.POINTER(vp)]
    L.gpugo_engine_destroy.argtypes = [vp]
    # output buffers by address (double* in the header): an engine admits thousands of problems
    L.gpugo_submit.argtypes = [vp, ctypes.POINTER(Spec), vp, vp, ctypes.c_int64, vp, ctypes.POINTER(Trace), _i64p]
    L.gpugo_submit_batch.argtypes = [vp, vp, ctypes.c_int64, vp, vp, ctypes.c_int64, vp, vp, _i64p]
    L.gpugo_run.argtypes = [vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]
    L.gpugo_poll.argtypes = [vp, ctypes.POINTER(Done), ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    L.gpugo_engine_free_bytes.argtypes = [vp, _i64p]
    L.gpugo_instance_bytes.argtypes = [ctypes.POINTER(Spec), _i64p]
    L.gpugo_strerror.argtypes = [ctypes.c_int]
    L.gpugo_strerror.restype = ctypes.c_char_p
    L.gpugo_device_info.argtypes = [ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
    L.gpugo_engine_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.gpugo_fp64_peak.argtypes = [ctypes.c_int32, _dp, _dp]
    L.gpugo_combine.argtypes = [_dp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _dp, ctypes.c_int64, _i64p]
    L.gpugo_checkpoint.argtypes = [vp, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, _i64p]
    L.gpugo_checkpoint_check.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    L.gpugo_restore.argtypes = [vp, ctypes.c_void_p, ctypes.c_int64, _dp, _dp, ctypes.c_int64, _dp,
                                ctypes.POINTER(Trace), _i64p]
    _lib = L
    return L


def check(rc: int, what: str = "") -> int:
    if rc < 0:
        raise GpugoError(rc, what)
    return rc
