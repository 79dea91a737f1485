"""Interval library of the oracle: directed rounding, endpoint functions, containment."""
import math
from fractions import Fraction as F

import mpmath as mp
import numpy as np
import pytest

mp.mp.prec = 200


def _exact_round(q, up):
    f = float(q)
    if F(f) == q:
        return f
    if up:
        return f if F(f) > q else float(np.nextafter(f, np.inf))
    return f if F(f) < q else float(np.nextafter(f, -np.inf))


def _values(rng, m):
    mags = 10.0 ** rng.integers(-320, 300, m)
    v = rng.normal(size=m) * mags
    extra = np.array([0.0, -0.0, 5e-324, -5e-324, 2.5e-323, 1e-310, -1e-310, 1.0, -1.0, 3.0])
    return np.concatenate([v, extra])


@pytest.mark.parametrize("op", ["add", "mul", "div"])
def test_directed_rounding_exact(oracle_lib, op):
    rng = np.random.default_rng(7)
    vals = _values(rng, 600)
    a = rng.choice(vals, 4000)
    b = rng.choice(vals, 4000)
    if op == "div":
        b[b == 0] = 1.5
    lo = oracle_lib.round_op(op, "down", a, b)
    hi = oracle_lib.round_op(op, "up", a, b)
    for x, y, l, h in zip(a, b, lo, hi):
        q = {"add": lambda: F(x) + F(y), "mul": lambda: F(x) * F(y), "div": lambda: F(x) / F(y)}[op]()
        if abs(q) > F(1.7976931348623157e308):
            continue
        assert l == _exact_round(q, False), (op, x, y)
        assert h == _exact_round(q, True), (op, x, y)


def test_directed_sqrt(oracle_lib):
    rng = np.random.default_rng(8)
    x = np.abs(_values(rng, 800))
    lo = oracle_lib.round_op("sqrt", "down", x)
    hi = oracle_lib.round_op("sqrt", "up", x)
    for v, l, h in zip(x, lo, hi):
        assert F(l) ** 2 <= F(v) <= F(h) ** 2
        assert h == l or h == np.nextafter(l, np.inf)


def _ulp_errors(fn, x, ref):
    y = oracle_lib_point(fn, x)
    out = []
    for xi, yi in zip(x, y):
        t = ref(mp.mpf(float(xi)))
        u = math.ulp(float(t)) if t != 0 else 5e-324
        out.append(float(abs(mp.mpf(float(yi)) - t) / u))
    return np.array(out)


oracle_lib_point = None


@pytest.fixture(autouse=True)
def _bind(oracle_lib):
    global oracle_lib_point
    oracle_lib_point = oracle_lib.point_fn


def test_exp_accuracy():
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.uniform(-744, 709.7, 3000), rng.uniform(-1, 1, 3000), rng.uniform(-40, 40, 3000)])
    assert _ulp_errors("exp", x, mp.exp).max() < 1.0


@pytest.mark.parametrize("fn,ref", [("sin", mp.sin), ("cos", mp.cos)])
def test_trig_accuracy(fn, ref):
    rng = np.random.default_rng(10)
    k = rng.integers(-2_000_000, 2_000_000, 1500)
    near = np.array([float(mp.mpf(int(kk)) * mp.pi / 2) for kk in k])
    x = np.concatenate([rng.uniform(-4e6, 4e6, 3000), rng.uniform(-10, 10, 3000), near,
                        np.nextafter(near, np.inf), rng.uniform(-1e-3, 1e-3, 500)])
    assert _ulp_errors(fn, x, ref).max() < 1.2


def _rand_intervals(rng, m, scale):
    a = rng.normal(size=m) * scale
    w = np.abs(rng.normal(size=m)) * scale * 10.0 ** rng.integers(-12, 1, m)
    return np.stack([a, a + w], axis=1)


def _contains(iv, x):
    return mp.mpf(float(iv[0])) <= x <= mp.mpf(float(iv[1]))


@pytest.mark.parametrize("op", ["add", "minus", "mul", "div", "sqr", "sqrt", "exp", "sin", "cos", "times", "plus"])
def test_interval_containment(oracle_lib, op):
    rng = np.random.default_rng(abs(hash(op)) % 2 ** 32)
    m = 300
    A = _rand_intervals(rng, m, 10.0)
    B = _rand_intervals(rng, m, 10.0)
    if op == "sqrt":
        A = np.abs(A); A.sort(axis=1)
    if op == "exp":
        A = A / 5
    if op in ("times", "plus"):
        B[:, 1] = B[:, 0]
    R = oracle_lib.ia_op(op, A, B)
    fns = {"add": lambda x, y: x + y, "minus": lambda x, y: x - y, "mul": lambda x, y: x * y,
           "div": lambda x, y: x / y, "sqr": lambda x, y: x * x, "sqrt": lambda x, y: mp.sqrt(x),
           "exp": lambda x, y: mp.exp(x), "sin": lambda x, y: mp.sin(x), "cos": lambda x, y: mp.cos(x),
           "times": lambda x, y: x * y, "plus": lambda x, y: x + y}
    for t in range(m):
        a, b, r = A[t], B[t], R[t]
        assert r[0] <= r[1] or (np.isnan(r[0]) and np.isnan(r[1]))
        if op == "div" and b[0] <= 0 <= b[1]:
            continue
        for _ in range(6):
            x = mp.mpf(float(a[0])) + (mp.mpf(float(a[1])) - mp.mpf(float(a[0]))) * mp.rand()
            y = mp.mpf(float(b[0])) + (mp.mpf(float(b[1])) - mp.mpf(float(b[0]))) * mp.rand()
            assert _contains(r, fns[op](x, y)), (op, a, b, r)
        for x in (mp.mpf(float(a[0])), mp.mpf(float(a[1]))):
            y = mp.mpf(float(b[0]))
            assert _contains(r, fns[op](x, y)), (op, a, b, r)


@pytest.mark.parametrize("op,ext", [("sin", [1, -1]), ("cos", [1, -1])])
def test_trig_extrema(oracle_lib, op, ext):
    """Intervals straddling k*pi/2 must reach the +-1 extrema (IA.py:441-444, :525-528)."""
    ks = np.arange(-40, 40)
    c = ks * (np.pi / 2)
    A = np.stack([c - 1e-3, c + 1e-3], axis=1)
    R = oracle_lib.ia_op(op, A)
    for k, r in zip(ks, R):
        v = float(getattr(mp, op)(mp.mpf(int(k)) * mp.pi / 2))
        if abs(v) == 1:
            assert (r[1] == 1.0) if v > 0 else (r[0] == -1.0)


def test_bump_and_zero_rules(oracle_lib):
    """power(.,2) of [0, x] widens its lower end below zero by 5 subnormal ulps (IA.py:267-279)."""
    r = oracle_lib.ia_op("sqr", np.array([[0.0, 2.0], [-0.0, 2.0], [-1.0, 2.0]]))
    assert r[0, 0] == -2.5e-323 and r[1, 0] == -2.5e-323 and r[2, 0] == 0.0
    assert r[2, 1] > 4.0 and r[2, 1] == np.nextafter(4.0, 10) + 4 * 8.881784197001252e-16
    e = oracle_lib.ia_op("exp", np.array([[-800.0, 0.0], [0.0, 800.0]]))
    assert e[0, 0] == 0.0 and e[1, 1] == np.inf
