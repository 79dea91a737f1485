"""The library's input checks against the oracle's: code lists with damaged
words, and problem descriptions with limits crossed.

The device interpreter checks no index: ``gpugo_instance_bytes`` (and every
entry point that takes a problem) must reject each array the interpreter could
not run within bounds.  The oracle carries its own, separately written checks
and runs every array it accepts.  Here thousands of compiled objectives with
one or two integer words changed (registers, coordinates, offsets, ranges,
opcodes, table and section fields) go to both: they must accept and reject the
same arrays, and the oracle must evaluate every accepted one (value, sample and
derivative lists) without failing.  No GPU is needed: the library validates on
the host.
"""
import ctypes

import numpy as np
import pytest

from gpugo_gb300 import codelist as CL
from gpugo_gb300 import objectives as O
from gpugo_gb300 import problems as P


@pytest.fixture(scope="module")
def lib():
    from gpugo_gb300 import _lib, build
    build.build()
    return _lib.load()


def _objectives():
    out = []
    for name in sorted(O.REFERENCE):
        for n in (6, 13):
            f, g, dom = O.REFERENCE[name](n)
            out.append((n, dom, CL.compile_objective(f, n, g).coef))
            out.append((n, dom, CL.compile_objective(f, n, "auto").coef))
            out.append((n, dom, CL.compile_objective(f, n, g, tables=False).coef))
    return out


def _damage(rng, coef, n):
    """One or two integer words of the array replaced by a value that is near
    a valid one (small numbers, +-1, +-n), a negative 32-bit number, one byte
    of a packed instruction word, a flipped bit or anything at all."""
    p = CL.parse(coef)
    U = CL.HEADER + CL.SEC_WORDS * len(p["sections"])
    I = U + CL.TAB_WORDS * len(p["tables"])
    C = I + CL.INS_WORDS * len(p["instructions"])
    c = coef.copy()
    w = c.view(np.uint64)
    for _ in range(1 + int(rng.random() < 0.25)):
        k = int(rng.integers(0, C))
        old = int(w[k])
        kind = int(rng.integers(6))
        if kind == 0:
            v = int(rng.integers(0, 20))
        elif kind == 1:
            v = (old + int(rng.choice([-1, 1, -n, n, n + 1]))) & 0xFFFFFFFF
        elif kind == 2:
            v = int(rng.integers(0, 1 << 32))
        elif kind == 3:
            b = int(rng.integers(4))
            v = (old & ~(0xFF << (8 * b))) | (int(rng.integers(0, 24)) << (8 * b))
        elif kind == 4:
            v = (-int(rng.integers(1, 4))) & 0xFFFFFFFF
        else:
            v = old ^ (1 << int(rng.integers(0, 32)))
        w[k] = v
    return c


@pytest.mark.parametrize("seed", [0, 1])
def test_library_and_oracle_accept_the_same_arrays(lib, oracle_lib, seed):
    from gpugo_gb300 import _spec
    objs = _objectives()
    rng = np.random.default_rng(0x66757A7A + seed)
    codes = np.array([0, 1, 3, 7], dtype=np.uint64)
    accepted = 0
    for t in range(5000):
        n, dom, coef = objs[int(rng.integers(len(objs)))]
        q = P.Problem(P.CODELIST, n, np.tile(dom, n), _damage(rng, coef, n), wid=2, group=3)
        s, keep = _spec(q)
        nbytes = ctypes.c_int64(0)
        lib_ok = lib.gpugo_instance_bytes(ctypes.byref(s), ctypes.byref(nbytes)) == 0
        try:
            lb, samp, _, _ = oracle_lib.eval_children(q, q.domain, 1, codes, 1e300)
            oracle_ok = True
        except ValueError:
            oracle_ok = False
        assert lib_ok == oracle_ok, (t, n, lib_ok)
        accepted += lib_ok
    # both kinds of outcome are exercised
    assert 500 < accepted < 4500


@pytest.mark.parametrize("seed", [0, 1])
def test_library_and_oracle_accept_the_same_specs(lib, oracle_lib, seed):
    """Problem descriptions of the four built-in families with limits crossed
    (dimension, split, samples, stop rule, coefficient count and signs, empty or
    NaN domain intervals): the library and the oracle accept the same ones.  One
    limit is the library's own: the chained family's gradient table holds wid^3
    entries per coordinate, so it takes at most 64 parts (the oracle has no
    tables)."""
    from gpugo_gb300 import _spec
    rng = np.random.default_rng(0x73706563 + seed)
    need = {P.COSQUAD: lambda n: 3 * n, P.CHAINED: lambda n: 2 * n - 2, P.EXPSQRT: lambda n: 2 + n,
            P.PRODCOS: lambda n: 1}
    accepted = 0
    for t in range(1500):
        # a valid description, then zero to two fields moved to a boundary value
        fam = int(rng.integers(1, 5))
        n = int(rng.integers(2, 64))
        wid, group, samples, stop = int(rng.integers(2, 6)), int(rng.integers(1, 11)), 10, 1
        for _ in range(int(rng.integers(0, 3))):
            f = int(rng.integers(6))
            if f == 0:
                fam = int(rng.choice([0, 5, 6, 1, 2]))
            elif f == 1:
                n = int(rng.choice([1, 2, 3, 50, 16384, 16385]))
            elif f == 2:
                wid = int(rng.choice([0, 1, 2, 64, 65, 65536]))
            elif f == 3:
                group = int(rng.choice([-1, 0, 1, 32, 33]))
            elif f == 4:
                samples = int(rng.choice([-1, 0, 1, 255, 256]))
            else:
                stop = int(rng.choice([-1, 0, 2]))
        ncoef = max(0, need.get(fam, lambda n: 4)(n) + int(rng.choice([0, 0, 0, -1, 1])))
        dom = np.tile([-1.0, 2.0], n)
        if rng.random() < 0.1:
            j = int(rng.integers(n))
            dom[2 * j], dom[2 * j + 1] = 2.0, -1.0
        if rng.random() < 0.05:
            dom[int(rng.integers(2 * n))] = np.nan
        coef = rng.uniform(0.5, 2.0, ncoef) * (-1.0 if rng.random() < 0.05 else 1.0)
        p = P.Problem(fam, n, dom, coef, wid=wid, group=group, samples=samples, stop_mode=stop)
        s, keep = _spec(p)
        nbytes = ctypes.c_int64(0)
        lib_ok = lib.gpugo_instance_bytes(ctypes.byref(s), ctypes.byref(nbytes)) == 0
        try:
            oracle_lib.eval_children(p, p.domain, 1, np.zeros(1, dtype=np.uint64), 1e300)
            oracle_ok = True
        except ValueError:
            oracle_ok = False
        if fam == P.CHAINED and wid > 64 and oracle_ok:
            assert not lib_ok
            continue
        assert lib_ok == oracle_ok, (t, fam, n, wid, group, samples, stop, ncoef)
        accepted += lib_ok
    assert 300 < accepted < 1300
