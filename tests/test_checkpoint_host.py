"""Checkpoint buffers checked on the host (``gpugo_checkpoint_check``, the checks
``gpugo_restore`` runs before it admits a solve).

The kernels index the parent table and the list with what a restored buffer
holds, so a damaged buffer must be refused before it reaches the device.  The
buffers here are built by hand in the library's checkpoint layout (a header with
the problem and the solve's state, then the domain, coefficients, parent rows,
their part widths and cycles, the list, emitted boxes and trace); real ones come
from ``Engine.checkpoint`` in the GPU tests.  No device is needed.
"""
import ctypes

import numpy as np
import pytest

import gpugo_gb300 as G
from gpugo_gb300 import problems as P

ST_EXPAND, ST_REPOP, ST_DONE = 1, 2, 3


class State(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("outcome", ctypes.c_int), ("cur", ctypes.c_int), ("cyc", ctypes.c_int),
                ("iter", ctypes.c_int64), ("ub", ctypes.c_uint64), ("ub_start", ctypes.c_uint64),
                ("ub_who", ctypes.c_uint64), ("count", ctypes.c_int64), ("count_new", ctypes.c_int64),
                ("count_before", ctypes.c_int64), ("removed_new", ctypes.c_int64), ("out_count", ctypes.c_int64),
                ("out_lb_min", ctypes.c_double), ("bounded", ctypes.c_int64), ("samples", ctypes.c_int64),
                ("ubc_count", ctypes.c_int64), ("m_children", ctypes.c_int64), ("b_done", ctypes.c_int64),
                ("seed_key", ctypes.c_uint64), ("cand_total", ctypes.c_int64), ("cand_done", ctypes.c_int64),
                ("has_who", ctypes.c_int), ("pad", ctypes.c_int), ("lb_max", ctypes.c_uint64)]


class Header(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_char * 8), ("family", ctypes.c_int32), ("n", ctypes.c_int32),
                ("wid", ctypes.c_int32), ("group", ctypes.c_int32), ("samples", ctypes.c_int32),
                ("stop_mode", ctypes.c_int32), ("width_tol", ctypes.c_double), ("gap_tol", ctypes.c_double),
                ("ub_init", ctypes.c_double), ("ncoef", ctypes.c_int64), ("max_iter", ctypes.c_int64),
                ("pool_cap", ctypes.c_int64), ("parent_cap", ctypes.c_int64), ("st", State),
                ("rows", ctypes.c_int64), ("cnt", ctypes.c_int64), ("nout", ctypes.c_int64),
                ("ntrace", ctypes.c_int64)]


def _pad8(b):
    return (b + 7) & ~7


@pytest.fixture(scope="module")
def lib():
    from gpugo_gb300 import build
    build.build()
    return G._lib.load()


def _checkpoint(p, rows=2, keys=None, out_keys=(), pcyc=None, **state):
    """A checkpoint of ``p`` after ``rows - 1`` expansions, in the library's layout."""
    n = p.n
    h = Header()
    h.magic = b"GPUGOCK2"
    h.family, h.n, h.wid, h.group, h.samples, h.stop_mode = p.family, n, p.wid, p.group, p.samples, p.stop_mode
    h.width_tol, h.gap_tol, h.ub_init = p.width_tol, p.gap_tol, 1e6
    h.ncoef = p.coef.size
    pcyc = [1] * rows if pcyc is None else list(pcyc)
    keys = [(0, 5), (rows - 1, 17), (rows - 1, 0)] if keys is None else list(keys)
    st = h.st
    st.status, st.cyc, st.iter = ST_EXPAND, pcyc[-1], rows - 1
    st.m_children = p.wid ** min(p.group, n - st.cyc + 1)
    st.count, st.count_before, st.out_count = len(keys), len(keys), len(out_keys)
    st.seed_key = (1 << 64) - 1
    st.out_lb_min = np.inf
    for k, v in state.items():
        setattr(st, k, v)
    h.rows, h.cnt, h.nout, h.ntrace = rows, len(keys), len(out_keys), 0
    par = np.tile(p.domain, rows)
    pw = np.tile((p.domain[1::2] - p.domain[0::2]) / p.wid, rows)
    cyc = np.zeros(_pad8(4 * rows) // 4, dtype=np.int32)
    cyc[:rows] = pcyc
    kk = np.array([(r << 32) | c for r, c in keys], dtype=np.uint64)
    ok = np.array([(r << 32) | c for r, c in out_keys], dtype=np.uint64)
    body = [p.domain, p.coef, par, pw, cyc, np.zeros(len(keys)), kk, ok, np.zeros(len(out_keys))]
    head = bytes(h) + b"\0" * (_pad8(ctypes.sizeof(h)) - ctypes.sizeof(h))
    return head + b"".join(np.ascontiguousarray(a).tobytes() for a in body)


def _ok(lib, data):
    buf = ctypes.create_string_buffer(data, len(data))
    return lib.gpugo_checkpoint_check(buf, len(data)) == 0


def test_layout_matches_the_library():
    assert ctypes.sizeof(State) == 176


@pytest.mark.parametrize("make", [lambda: P.config1(), lambda: P.config2(),
                                  lambda: P.instance(P.PRODCOS, 13, 5, 1e-6)])
def test_well_formed_checkpoints_pass(lib, make):
    p = make()
    c2 = 1 + p.group if p.group < p.n else 1
    assert _ok(lib, _checkpoint(p))
    assert _ok(lib, _checkpoint(p, rows=3, pcyc=[1, c2, 1], out_keys=[(1, 3)]))
    assert _ok(lib, _checkpoint(p, rows=1, keys=[], status=ST_DONE))
    assert G.checkpoint_ok(_checkpoint(p))


def test_damaged_checkpoints_are_refused(lib):
    p = P.instance(P.PRODCOS, 13, 5, 1e-6)          # split groups of 8 over 13 coordinates: cycles 1 and 9
    assert p.group == 8 and p.n == 13
    m1 = p.wid ** 8
    good = _checkpoint(p, rows=3, pcyc=[1, 9, 1], keys=[(0, 1), (1, p.wid ** 5 - 1), (2, m1 - 1)])
    assert _ok(lib, good)
    bad = {
        "status": dict(status=0), "status high": dict(status=4),
        "cycle 0": dict(cyc=0), "cycle past n": dict(cyc=14),
        "iteration vs rows": dict(iter=5), "children of the cycle": dict(m_children=m1 + 1),
        "list count before": dict(count_before=4), "negative counter": dict(ubc_count=-1),
        "emitted count": dict(out_count=-1), "sample index": dict(has_who=1, ub_who=(1 << 40) | (2 << 8) | 10),
    }
    for name, st in bad.items():
        data = _checkpoint(p, rows=3, pcyc=[1, 9, 1], keys=[(0, 1), (1, 2), (2, 3)], **st)
        assert not _ok(lib, data), name
    # list entries: a row past the parent table, a code past its parent's children
    assert not _ok(lib, _checkpoint(p, rows=3, pcyc=[1, 9, 1], keys=[(3, 0)]))
    assert not _ok(lib, _checkpoint(p, rows=3, pcyc=[1, 9, 1], keys=[(1, p.wid ** 5)]))
    assert not _ok(lib, _checkpoint(p, rows=3, pcyc=[1, 9, 1], out_keys=[(2, m1)]))
    # parent cycles outside 1..n
    assert not _ok(lib, _checkpoint(p, rows=3, pcyc=[1, 0, 1]))
    assert not _ok(lib, _checkpoint(p, rows=3, pcyc=[1, 14, 1]))
    # truncated, wrong magic, counts larger than the buffer, a bad problem
    assert not _ok(lib, good[:-8])
    assert not _ok(lib, good[:100])
    assert not _ok(lib, b"X" + good[1:])
    h = Header.from_buffer_copy(good)
    for field, v in (("rows", 1 << 40), ("cnt", 1 << 40), ("nout", 1 << 60), ("ntrace", 1 << 59),
                     ("ncoef", -1), ("n", 16385), ("wid", 1)):
        g = Header.from_buffer_copy(good)
        setattr(g, field, v)
        assert not _ok(lib, bytes(g) + good[ctypes.sizeof(h):]), field
    dom_at = _pad8(ctypes.sizeof(h))
    flipped = bytearray(good)
    flipped[dom_at:dom_at + 16] = np.array([1.0, -1.0]).tobytes()   # lo > hi
    assert not _ok(lib, bytes(flipped))
    assert not G.checkpoint_ok(good[:-8])
