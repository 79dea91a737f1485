"""The C-ABI library loads and exports every entry point include/gpugo.h declares.

No compute call is made here: this runs without a GPU.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "gpugo.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gpugo_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from gpugo_gb300 import _lib, build
    build.build()
    return _lib.load()


def test_exports_match_header(lib):
    from gpugo_gb300 import _lib
    declared = _declared()
    assert declared, "no declarations found"
    assert sorted(_lib.EXPORTS) == declared
    for name in declared:
        assert hasattr(lib, name), name


def test_strerror(lib):
    assert lib.gpugo_strerror(0) == b"ok"
    assert lib.gpugo_strerror(-4) == b"box pool capacity exceeded"


def test_instance_bytes_validates(lib):
    import numpy as np
    import gpugo_gb300 as G
    p = G.config2()
    assert G.instance_bytes(p) > 0
    bad = G.config2()
    bad.domain[0], bad.domain[1] = 1.0, -1.0
    with pytest.raises(G.GpugoError):
        G.instance_bytes(bad)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from gpugo_gb300 import _lib, build
    monkeypatch.delenv("GPUGO_LIB", raising=False)
    monkeypatch.setattr(build, "LIB", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError):
        _lib.load()
    monkeypatch.setenv("GPUGO_LIB", str(tmp_path / "other.so"))   # a named build that is not there
    with pytest.raises(ImportError):
        _lib.load()


def test_solve_record_is_json_ready():
    import json
    import numpy as np
    import gpugo_gb300 as G
    r = G.SolveResult(lb=-1.0, ub=-0.5, status=G.CERTIFIED, iterations=3, boxes_bounded=30, samples_evaluated=12,
                      pool_size=2, n_boxes=2, boxes=np.zeros((2, 1, 2)), box_lbs=np.zeros(2), xhat=None,
                      device_ms=0.25, trace={"n_surv": np.array([4, 2, 1]), "pool": np.array([4, 5, 2])})
    rec = json.loads(json.dumps(r.record("t")))
    assert rec["gap"] == 0.5 and rec["certified"] and rec["survivors"] == [4, 2, 1] and rec["list_sizes"] == [4, 5, 2]


def test_spec_validation_on_the_host(lib):
    """gpugo_instance_bytes validates a problem without touching the device:
    the dimension limit (16384, above the reference's largest script), split
    limits, and that a code list is compiled for the problem's n."""
    import numpy as np
    import gpugo_gb300 as G
    from gpugo_gb300 import objectives as O
    from gpugo_gb300 import problems as P

    def accepts(p):
        s, keep = G._spec(p)
        out = ctypes.c_int64(0)
        rc = lib.gpugo_instance_bytes(ctypes.byref(s), ctypes.byref(out))
        return rc == 0, out.value

    def cosquad(n):
        return P.Problem(P.COSQUAD, n, np.tile([-1.0, 1.0], n), np.ones(3 * n), wid=3, group=4)

    ok, nbytes = accepts(cosquad(16384))
    assert ok and nbytes > 0
    assert not accepts(cosquad(16385))[0]
    p = cosquad(40)
    p.wid, p.group = 2, 33          # 2^33 children per iteration (the group is capped by n)
    assert not accepts(p)[0]
    p.wid, p.group = 2, 32          # 2^32: the largest split
    assert accepts(p)[0]
    lv = O.problem("levy", 6)
    assert accepts(lv)[0]
    wrong_n = P.Problem(P.CODELIST, 7, np.tile([-10.0, 10.0], 7), lv.coef, wid=3, group=7)
    assert not accepts(wrong_n)[0]


def test_null_arguments_are_rejected_before_the_device(lib):
    """Missing output buffers, a null engine or a null problem give
    GPUGO_ERR_INVALID from the host checks (no device is touched, so this runs
    without a GPU)."""
    import numpy as np
    import gpugo_gb300 as G
    INVALID = -1
    p = G.config2()
    s, keep = G._spec(p)
    codes = np.zeros(4, dtype=np.uint64)
    out = np.zeros(4)
    flags = np.zeros(4, dtype=np.int32)
    dp = ctypes.POINTER(ctypes.c_double)
    box = p.domain.ctypes.data_as(dp)
    cp = codes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    fp = flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    for fn in (lib.gpugo_eval_children, lib.gpugo_eval_children_static):
        assert fn(ctypes.byref(s), box, 1, cp, 4, 1e300, None, out.ctypes.data_as(dp), fp) == INVALID
        assert fn(ctypes.byref(s), box, 1, cp, 4, 1e300, out.ctypes.data_as(dp), None, fp) == INVALID
        assert fn(ctypes.byref(s), box, 1, cp, 4, 1e300, out.ctypes.data_as(dp), out.ctypes.data_as(dp),
                  None) == INVALID
        assert fn(ctypes.byref(s), None, 1, cp, 4, 1e300, out.ctypes.data_as(dp), out.ctypes.data_as(dp),
                  fp) == INVALID
        assert fn(ctypes.byref(s), box, 0, cp, 4, 1e300, out.ctypes.data_as(dp), out.ctypes.data_as(dp),
                  fp) == INVALID                       # cycles are 1-based
        assert fn(None, box, 1, cp, 4, 1e300, out.ctypes.data_as(dp), out.ctypes.data_as(dp), fp) == INVALID
    assert lib.gpugo_instance_bytes(ctypes.byref(s), None) == INVALID
    assert lib.gpugo_instance_bytes(None, ctypes.byref(ctypes.c_int64())) == INVALID
    n_done = ctypes.c_int32()
    assert lib.gpugo_poll(None, None, 0, ctypes.byref(n_done)) == INVALID
    assert lib.gpugo_run(None, 1, None) == INVALID
    assert lib.gpugo_solve(ctypes.byref(s), None, None, None, 0, None, None) == INVALID
    res = G._lib.Result()
    assert lib.gpugo_solve(ctypes.byref(s), ctypes.byref(res), None, None, (1 << 40) + 1, None, None) == INVALID
    tr = G._lib.Trace(16, None, None, None, None)          # rows promised, no arrays
    assert lib.gpugo_solve(ctypes.byref(s), ctypes.byref(res), None, None, 4, None, ctypes.byref(tr)) == INVALID
    adm = ctypes.c_int64(-5)
    tk = np.zeros(2, dtype=np.int64)
    assert lib.gpugo_submit_batch(None, ctypes.byref(s), 1, None, None, 0, None, tk.ctypes.data,
                                  ctypes.byref(adm)) == INVALID
    assert lib.gpugo_submit_batch(None, None, 0, None, None, 0, None, None, None) == INVALID
    nr = ctypes.c_int64()
    assert lib.gpugo_combine(None, 3, 2, 1e-3, None, 0, ctypes.byref(nr)) == INVALID
    assert lib.gpugo_combine(out.ctypes.data_as(dp), 1, 2, -1.0, None, 0, ctypes.byref(nr)) == INVALID


def test_python_side_checks_array_sizes(lib):
    """The C ABI reads 2n bounds through plain pointers: the Python mirror
    refuses a domain or a parent box of the wrong size before the call (for a
    batch admission, before anything is admitted)."""
    import numpy as np
    import gpugo_gb300 as G
    p = G.config2()
    p.domain = p.domain[:-2]                  # changed after construction
    with pytest.raises(ValueError):
        G._spec(p)

    class NoEngine:                           # a call would fail: there is none
        def __getattr__(self, name):
            raise AssertionError(f"{name} called")
    e = object.__new__(G.Engine)
    e._L, e._h, e._pending = NoEngine(), None, {}
    with pytest.raises(ValueError, match="problem 1"):
        e.submit_many([G.config2(), p, G.config2()], box_cap=2)
    assert e._pending == {}
    q = G.config2()
    with pytest.raises(ValueError):
        G.eval_children(q, q.domain[:6], 1, np.zeros(2, dtype=np.uint64), 1e300)


def test_integration_binding_matches_the_library(lib, monkeypatch):
    """The ctypes binding shown to reference maintainers
    declares the same structures as the library, and its rastrigin50.py spec
    passes the library's checks (the solve itself needs a GPU)."""
    import gpugo_gb300 as G
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = text.split("## 2. Python binding", 1)[1].split("```python", 1)[1].split("```", 1)[0]
    setup = block.split("rc = lib.gpugo_solve", 1)[0]
    monkeypatch.chdir(ROOT)
    ns = {}
    exec(compile(setup, "INTEGRATION.md", "exec"), ns)
    for mine, theirs in ((ns["Spec"], G._lib.Spec), (ns["Result"], G._lib.Result)):
        assert ctypes.sizeof(mine) == ctypes.sizeof(theirs)
        assert [f[0] for f in mine._fields_] == [f[0] for f in theirs._fields_]
        for (a, ta), (b, tb) in zip(mine._fields_, theirs._fields_):
            assert getattr(mine, a).offset == getattr(theirs, b).offset, a
    out = ctypes.c_int64()
    assert lib.gpugo_instance_bytes(ctypes.cast(ctypes.byref(ns["spec"]), ctypes.POINTER(G._lib.Spec)),
                                    ctypes.byref(out)) == 0 and out.value > 0


def _eval_rc(lib, fn, p, codes, cyc=1):
    import numpy as np
    import gpugo_gb300 as G
    s, keep = G._spec(p)
    codes = np.ascontiguousarray(codes, dtype=np.uint64)
    m = codes.size
    out = np.zeros(max(m, 1))
    flags = np.zeros(max(m, 1), dtype=np.int32)
    dp = ctypes.POINTER(ctypes.c_double)
    return getattr(lib, fn)(ctypes.byref(s), p.domain.ctypes.data_as(dp), cyc,
                            codes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), m, 1e300,
                            out.ctypes.data_as(dp), out.ctypes.data_as(dp),
                            flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))


# Largest child-code count gpugo_eval_children_static takes for the 8-variable
# chained instance (wid 4): its descriptor, instance region and 28 bytes per code
# in 256-byte aligned pieces fill the 8 MiB scratch.
STATIC_MAX_CODES_CHAINED8 = 296_672


def test_child_codes_are_checked_unsigned_before_the_device(lib):
    """A child code is an index in [0, wid^g).  Codes of 2^63 and above (negative
    as signed integers) and codes at wid^g are refused by both eval entry
    points with GPUGO_ERR_INVALID, on the host, before the device is queried
    (the reference refuses indices outside its child grid, ackley50.py:532-540).
    wid = 3 is not a power of two: there the digit packing of an out-of-range
    code would give digits >= wid."""
    import gpugo_gb300 as G
    from gpugo_gb300 import problems as P
    INVALID = -1
    q = P.instance(P.COSQUAD, 5, 3, split=(3, 5))
    M = 3 ** 5
    for fn in ("gpugo_eval_children", "gpugo_eval_children_static"):
        for bad in (1 << 63, (1 << 64) - 1, M, 1 << 32):
            assert _eval_rc(lib, fn, q, [0, bad, 1]) == INVALID, (fn, bad)
        assert _eval_rc(lib, fn, q, [0, M - 1]) != INVALID
        # a short last cycle has fewer children: codes are checked against them
        assert _eval_rc(lib, fn, G.config2(), [4 ** 7], cyc=2) == INVALID
        assert _eval_rc(lib, fn, G.config2(), [4 ** 7 - 1], cyc=2) != INVALID


def test_static_scratch_limit_is_checked_on_the_host(lib):
    """gpugo_eval_children_static refuses a request larger than its scratch
    (GPUGO_ERR_SCRATCH_LIMIT) before it scans the codes or queries a device;
    the boundary is exact: one code fewer is accepted."""
    import numpy as np
    import gpugo_gb300 as G
    p = G.config2()
    m = STATIC_MAX_CODES_CHAINED8
    assert _eval_rc(lib, "gpugo_eval_children_static", p, np.zeros(m + 1)) == -10
    assert _eval_rc(lib, "gpugo_eval_children_static", p, np.zeros(m)) != -10
    # an oversize request with invalid codes is still a scratch-limit refusal
    assert _eval_rc(lib, "gpugo_eval_children_static", p, np.full(m + 1, 1 << 63)) == -10
    # the allocating entry point has no such limit
    assert _eval_rc(lib, "gpugo_eval_children", p, np.zeros(m + 1)) != -10
