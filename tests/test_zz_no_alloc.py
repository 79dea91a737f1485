"""gpugo_eval_children_static: the bound/prune pass for callers that cannot
allocate device memory (hosts that own the whole device heap, or loops that
cannot afford cudaMalloc's device-wide synchronisation).

Its results must equal those of gpugo_eval_children, the allocating entry point,
on two calls in a row with different problems (the second call reuses the fixed
scratch the first one filled).  This file is collected last so that a failure
here does not hide the other tests in a run that stops at the first failure.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


def _call(L, fn, p, pbox, cyc, codes, ub):
    import gpugo_gb300 as G
    s, keep = G._spec(p)
    pb = np.ascontiguousarray(pbox, dtype=np.float64)
    codes = np.ascontiguousarray(codes, dtype=np.uint64)
    m = codes.size
    lb, samp, flag = np.empty(m), np.empty(m), np.empty(m, dtype=np.int32)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = getattr(L, fn)(ctypes.byref(s), pb.ctypes.data_as(dp), int(cyc),
                        codes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), m, float(ub),
                        lb.ctypes.data_as(dp), samp.ctypes.data_as(dp),
                        flag.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return rc, lb, samp, flag


def _same(a, b):
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.fixture(scope="module")
def lib():
    from gpugo_gb300 import _lib, build
    build.build()
    return _lib.load()


def test_static_matches_allocating_entry_point(lib):
    from gpugo_gb300 import problems as P
    rng = np.random.default_rng(11)
    g = np.load(GOLD)
    ref = P.Problem(1, 50, g["rastrigin_domain"], g["rastrigin_coef"], wid=4, group=10, samples=10,
                    stop_mode=P.STOP_WIDTH, width_tol=1e-4, ub_init=1e6)
    from gpugo_gb300 import objectives as O
    levy = O.problem("levy", 12, split=(4, 6))      # a code list: term and flag tables in the scratch
    cases = [
        (P.config2(), P.config2().domain, 1, rng.integers(0, 4 ** 8, 5000)),
        (ref, g["rastrigin_parents"][1], 11, rng.integers(0, 4 ** 10, 5000)),
        (levy, levy.domain, 7, rng.integers(0, 4 ** 6, 3000)),
    ]
    for p, pbox, cyc, codes in cases:  # two calls in a row on the shared scratch
        rc0, lb0, s0, f0 = _call(lib, "gpugo_eval_children", p, pbox, cyc, codes, 1e300)
        ub = float(np.quantile(lb0, 0.4))
        rc0, lb0, s0, f0 = _call(lib, "gpugo_eval_children", p, pbox, cyc, codes, ub)
        rc1, lb1, s1, f1 = _call(lib, "gpugo_eval_children_static", p, pbox, cyc, codes, ub)
        assert rc0 == 0 and rc1 == 0
        assert _same(lb1, lb0) and _same(s1, s0)
        np.testing.assert_array_equal(f1, f0)
        assert 0 < f1.sum() < f1.size


def test_static_rejects_oversize(lib):
    from gpugo_gb300 import problems as P
    p = P.config2()
    codes = np.zeros(1_000_000, dtype=np.uint64)   # 28 MB of codes and results > 8 MiB
    rc, *_ = _call(lib, "gpugo_eval_children_static", p, p.domain, 1, codes, 1e300)
    assert rc == -10
    assert lib.gpugo_strerror(rc).startswith(b"request exceeds the fixed scratch")


def test_static_at_the_scratch_boundary(lib):
    """The largest request that fits the scratch (every byte of the 8 MiB array
    in use) gives the allocating entry point's results bit for bit, twice in a
    row; one code more is refused."""
    from test_capi import STATIC_MAX_CODES_CHAINED8 as M
    from gpugo_gb300 import problems as P
    p = P.config2()
    rng = np.random.default_rng(5)
    codes = rng.integers(0, 4 ** 8, M).astype(np.uint64)
    rc0, lb0, s0, f0 = _call(lib, "gpugo_eval_children", p, p.domain, 1, codes, 1e300)
    ub = float(np.quantile(lb0, 0.3))
    rc0, lb0, s0, f0 = _call(lib, "gpugo_eval_children", p, p.domain, 1, codes, ub)
    assert rc0 == 0
    for _ in range(2):
        rc1, lb1, s1, f1 = _call(lib, "gpugo_eval_children_static", p, p.domain, 1, codes, ub)
        assert rc1 == 0
        assert _same(lb1, lb0) and _same(s1, s0)
        np.testing.assert_array_equal(f1, f0)
    rc2, *_ = _call(lib, "gpugo_eval_children_static", p, p.domain, 1, np.append(codes, codes[:1]), ub)
    assert rc2 == -10
