"""Random objectives through the front end (compiler, term tables, derived
gradients) on the oracle's interpreter: rigour checks that hold for any
objective.

* The LB of a child box lies below the objective at every point of the box
  (plain FP64 evaluation, with a rounding allowance).
* The smallest sampled upper bound lies above the objective at the sample
  points it came from (it is an upper bound of a value the box attains).
* A box that the derived KKT test rules out has a gradient component whose sign
  does not change over the box, and that component's face is not on the domain
  boundary: checked at random points of the box by central differences.
* Code compiled with and without term tables gives the same bits.
"""
import numpy as np
import pytest

from gpugo_gb300 import codelist as CL
from gpugo_gb300 import problems as P

X, Sum, Prod, sqr, sin, cos, exp, sqrt = CL.X, CL.Sum, CL.Prod, CL.sqr, CL.sin, CL.cos, CL.exp, CL.sqrt


def _unary(rng, e, depth):
    k = int(rng.integers(0, 7))
    c = float(rng.uniform(0.3, 2.0))
    if k == 0:
        return sqr(e) * c
    if k == 1:
        return sin(e * c)
    if k == 2:
        return cos(e * c) * c
    if k == 3:
        return exp(sin(e) * 0.5)              # bounded argument
    if k == 4:
        return sqrt(sqr(e) + c)
    if k == 5:
        return e / (sqr(e) + 1.0)             # positive denominator
    return e * c + (-c)


def _term(rng, xs, depth=2):
    """A random expression of the given coordinate expressions."""
    e = xs[int(rng.integers(0, len(xs)))]
    for _ in range(depth):
        e = _unary(rng, e, depth)
        if rng.random() < 0.4:
            other = xs[int(rng.integers(0, len(xs)))]
            op = int(rng.integers(0, 3))
            e = e + other * 0.7 if op == 0 else (e - sqr(other) * 0.3 if op == 1 else e * (sqr(other) * 0.1 + 1.0))
    return e


def _objective(rng, n):
    offs = [0] if rng.random() < 0.5 else [0, 1]
    hi = n - max(offs)
    body = lambda i: _term(rng_state(), [X[i + o] for o in offs])
    # the body lambda must give the same expression on every call: draw it once
    seed = int(rng.integers(1 << 30))

    def rng_state():
        return np.random.default_rng(seed)

    f = Sum(body, hi=hi)
    extra = rng.random()
    if extra < 0.25:        # a fixed coordinate inside the body
        f = Sum(lambda i: body(i) * (sqr(X[0]) * 0.1 + 1.0), hi=hi)
    elif extra < 0.5:       # a (loop-invariant) reduction inside the body
        f = Sum(lambda i: body(i) + sqr(X[i]) * Sum(lambda k: cos(X[k]) * 0.1), hi=hi)
    if rng.random() < 0.5:
        f = f + sqr(X[0] + (-0.5)) * 0.5
    if rng.random() < 0.3:
        f = f * 0.25 + Prod(lambda i: cos(X[i] * 0.2), init=1.0)
    return f


@pytest.mark.parametrize("seed", range(12))
def test_random_objectives_are_rigorous(oracle_lib, seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(2, 6))
    f = _objective(rng, n)
    lo, hi = -2.0, 2.5
    dom = np.tile([lo, hi], n)
    wid, group = 3, n
    coef_t = CL.compile_objective(f, n, "auto").coef
    coef_l = CL.compile_objective(f, n, "auto", tables=False).coef
    pt = P.Problem(P.CODELIST, n, dom, coef_t, wid=wid, group=group, samples=4)
    pl = P.Problem(P.CODELIST, n, dom, coef_l, wid=wid, group=group, samples=4)
    value = lambda x: CL.point_value(coef_l, x)
    pruned_seen = 0
    for trial in range(6):
        # a parent box somewhere in the domain (sometimes tiny, sometimes large)
        w = (hi - lo) * 10.0 ** rng.uniform(-4, -0.3, n)
        c = rng.uniform(lo, hi - w)
        pbox = np.empty(2 * n)
        pbox[0::2], pbox[1::2] = c, c + w
        codes = rng.integers(0, wid ** n, 40).astype(np.uint64)
        a = oracle_lib.eval_children(pt, pbox, 1, codes, 1e300)
        b = oracle_lib.eval_children(pl, pbox, 1, codes, 1e300)
        for u, v in zip(a, b):
            assert np.array_equal(np.asarray(u).view(np.uint8), np.asarray(v).view(np.uint8))
        lbs, samps, _, dflags = a
        for k, code in enumerate(codes):
            box = oracle_lib.child_box(pt, pbox, 1, int(code)).reshape(n, 2)
            pts = box[:, 0] + (box[:, 1] - box[:, 0]) * rng.random((8, n))
            vals = np.array([value(x) for x in pts])
            scale = 1.0 + np.max(np.abs(vals))
            assert np.all(lbs[k] <= vals + 1e-9 * scale), (seed, trial, k)
            # the sampled upper bound is attained at a diagonal point of the box
            S = 4
            diag = [box[:, 0] + (box[:, 1] - box[:, 0]) / (S + 1) * (j + 1) for j in range(S)]
            assert samps[k] >= min(value(x) for x in diag) - 1e-9 * scale
            if dflags[k]:
                pruned_seen += 1
                h = 1e-7 * np.maximum(1.0, np.abs(box[:, 1] - box[:, 0]))
                inner = box[:, 0] + (box[:, 1] - box[:, 0]) * (0.05 + 0.9 * rng.random((6, n)))
                grads = np.array([[(value(x + h[j] * e) - value(x - h[j] * e)) / (2 * h[j])
                                   for j, e in enumerate(np.eye(n))] for x in inner])
                signs_fixed = [j for j in range(n)
                               if (np.all(grads[:, j] > -1e-6) or np.all(grads[:, j] < 1e-6))]
                assert signs_fixed, (seed, trial, k, grads)
    assert pruned_seen > 0      # the derived KKT test was exercised
