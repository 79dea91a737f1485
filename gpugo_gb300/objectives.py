"""Objectives written as code lists (family ``CODELIST``).

Seven are the reference benchmarks that have no built-in family, each restating
the reference's own value, sample and derivative code lists operation by
operation (the sample list of every script is its value list run on the
diagonal points):

=============  ==========================================  ==================
objective      reference code lists                        domain
=============  ==========================================  ==================
levy           GPUGO_1.1/6-Levy/levy50.py:141-226, :382-563          [-10, 10]
salomon        GPUGO_1.1/8-Salomon/salomon50.py:112-197, :302-402    [-100, 110]
corrupted      GPUGO_1.1/9-Styblinski/corrupted50.py:115-208, :332-430  [-10, 11]
deflected      GPUGO_1.1/2-Belegundu/deflected50.py:113-207, :318-424   [-10, 11]
cosine         GPUGO_1.1/3-Breiman/cosine50.py:111-196, :302-377     [-1, 2]
trigonometric  GPUGO_1.1/4-Fu/trigonometric50.py:112-217, :342-443   [-10, 10]
sinusoidal     GPUGO_1.1/10-Zabinsky/sinusoidal50.py:113-202, :315-443  [0, pi]
=============  ==========================================  ==================

Two of the reference's lists are not restated as they are, because as written
they do not bound what they claim to bound:

* deflected50.py's derivative sums (x_k - 5)^2 for the coordinate k left over
  from the preceding loop instead of for every coordinate (:376-386); the code
  list here sums over all coordinates, which is the gradient of its value list.
* cosine50.py's sample list drops the sum of squares (:245-299), so its
  "upper bound" is not a value of the objective; the sample list here is the
  value list, as in every other script.

The other four (``cosquad``, ``chained``, ``expsqrt``, ``prodcos``) are the
built-in families restated as code lists.  They evaluate to the same bits as
the built-in kernels, which pins the code-list path to the built-in one.

Scalar constants are written as the reference writes them (``math.pi / 4``,
``(3 * math.pi) / 4``, ...), so they are the same doubles.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from .codelist import (Coef, Const, Gradient, Prod, Section, Sum, X, compile_objective, cos, exp, sin, sqr,
                       sqrt)
from .problems import CODELIST, STOP_GAP, Problem


# ---------------------------------------------------------------------------
# directed rounding of exact rationals (interval constants)
# ---------------------------------------------------------------------------
def _rd(q: Fraction) -> float:
    f = float(q)
    return f if Fraction(f) <= q else float(np.nextafter(f, -np.inf))


def _ru(q: Fraction) -> float:
    f = float(q)
    return f if Fraction(f) >= q else float(np.nextafter(f, np.inf))


def _sqrt_rd(x: float) -> float:
    r = math.sqrt(x)
    return r if Fraction(r) ** 2 <= Fraction(x) else float(np.nextafter(r, -np.inf))


def _sqrt_ru(x: float) -> float:
    r = math.sqrt(x)
    return r if Fraction(r) ** 2 >= Fraction(x) else float(np.nextafter(r, np.inf))


E_LO = float.fromhex("0x1.5bf0a8b145769p+1")   # RN(e) < e
E_HI = float(np.nextafter(E_LO, np.inf))


# ---------------------------------------------------------------------------
# the reference benchmarks without a built-in family
# ---------------------------------------------------------------------------
def levy(n: int):
    pi = math.pi
    head = sqr(X[-1] * (1 / 4) + (-1 / 4)) + 10 * sqr(sin(X[0] * (pi / 4) + (3 * pi) / 4))
    body = Sum(lambda i: sqr(X[i - 1] * (1 / 4) + (-1 / 4)) * (10 * sqr(sin(X[i] * (pi / 4) + (3 * pi) / 4)) + 1),
               lo=1)
    f = (body + head) * (pi / n)

    def tail(j):       # 10 sin^2(pi/4 x_{j+1} + 3pi/4) + 1
        return 10 * sqr(sin(X[j + 1] * (pi / 4) + (3 * pi) / 4)) + 1

    first = lambda j: (sin(X[j] * (pi / 2) + (3 * pi) / 2) * ((5 * pi) / 2)
                       + ((X[j] + (-1)) * tail(j)) * (1 / 8)) * (pi / n)
    mid = lambda j: ((sin(X[j] * (pi / 2) + (3 * pi) / 2) * sqr(X[j - 1] + (-1))) * ((5 * pi) / 32)
                     + ((X[j] + (-1)) * tail(j)) * (1 / 8)) * (pi / n)
    last = lambda j: ((X[j] + (-1)) * (1 / 8)
                      + (sin(X[j] * (pi / 2) + (3 * pi) / 2) * sqr(X[j - 1] + (-1))) * ((5 * pi) / 32)) * (pi / n)
    # the last test reads the bounds of x_{n-1}, as levy50.py:551-557 does
    secs = [Section(first, 0, 1)]
    if n > 2:
        secs.append(Section(mid, 1, n - 1))
    secs.append(Section(last, n - 1, n, check=-1))
    return f, Gradient(secs), (-10.0, 10.0)


def salomon(n: int):
    r = sqrt(Sum(lambda i: sqr(X[i])))
    f = (r * 0.1 - cos(r * (2 * math.pi))) + 1
    g = lambda j: ((sin(r * (2 * math.pi)) * X[j]) * (2 * math.pi) + X[j] * 0.1) / r
    return f, Gradient(g, skip_if_contains=0.0), (-100.0, 110.0)


def corrupted(n: int):
    f = Sum(lambda i: sqr(X[i])) * (1 / (2 * n)) + Prod(lambda i: cos(X[i]), init=float(-4 * n))
    P = Prod(lambda i: cos(X[i]), init=float(4 * n))
    q = lambda j: P / cos(X[j])
    g = lambda j: q(j) * sin(X[j]) + X[j] * (1 / n)
    return f, Gradient([Section(g, skip_infinite=q)]), (-10.0, 11.0)


def deflected(n: int):
    s = Sum(lambda i: sqr(X[i] + (-5)))
    f = s * 0.1 - cos(sqrt(s) * 5)
    r = sqrt(s)
    g = lambda j: (X[j] + (-5)) * 0.2 + ((sin(r * 5) * 5) * (X[j] + (-5))) / r
    return f, Gradient(g, skip_if_contains=5.0), (-10.0, 11.0)


def cosine(n: int):
    f = Sum(lambda i: cos(X[i] * (5 * math.pi))) * (-0.1) + Sum(lambda i: sqr(X[i]))
    g = lambda j: sin(X[j] * (5 * math.pi)) * (0.5 * math.pi) + X[j] * 2
    return f, Gradient(g), (-1.0, 2.0)


def trigonometric(n: int):
    def term(i):
        t = sqr(X[i] + (-0.9))
        return t + (sqr(sin(t * 14)) * 6 + sqr(sin(t * 7)) * 8)

    f = Sum(term) + 1

    def g(j):
        u = X[j] + (-0.9)
        a = sqr(u) * 7
        b = sqr(u) * 14
        return (((sin(a) * cos(a)) * u) * 224 + ((sin(b) * cos(b)) * u) * 336) + u * 2

    return f, Gradient(g), (-10.0, 10.0)


def sinusoidal(n: int):
    c = -math.pi / 6
    f = (Prod(lambda i: sin(X[i] + c), init=2.5) + Prod(lambda i: sin((X[i] + c) * 5), init=1.0)) * (-1)
    Q1 = Prod(lambda i: sin(X[i] + c), init=2.5)
    Q2 = Prod(lambda i: sin((X[i] + c) * 5), init=5.0)

    def g(j):
        d5 = X[j] + c
        d10 = d5 * 5
        return ((Q1 / sin(d5)) * cos(d5) + (Q2 / sin(d10)) * cos(d10)) * (-1)

    return f, Gradient(g), (0.0, math.pi)


REFERENCE = {"levy": levy, "salomon": salomon, "corrupted": corrupted, "deflected": deflected, "cosine": cosine,
             "trigonometric": trigonometric, "sinusoidal": sinusoidal}


# ---------------------------------------------------------------------------
# the built-in families as code lists
# ---------------------------------------------------------------------------
def cosquad(n: int, coef: np.ndarray):
    a, b, c = coef[:n], coef[n:2 * n], coef[2 * n:3 * n]
    K = Coef((2 * math.pi) * c)
    A, B, A2 = Coef(a), Coef(b), Coef(2.0 * a)
    f = Sum(lambda i: sqr(X[i]) * A[i] - cos(X[i] * K[i]) * B[i]) + Sum(lambda i: B[i])
    g = lambda j: X[j] * A2[j] + sin(X[j] * K[j]) * (B[j] * K[j])
    return f, Gradient(g)


def chained(n: int, coef: np.ndarray):
    p, q = coef[:n - 1], coef[n - 1:2 * n - 2]
    P, Q, P4, P2, Q2, M2Q = (Coef(v) for v in (p, q, 4.0 * p, 2.0 * p, 2.0 * q, -2.0 * q))
    f = Sum(lambda i: sqr(sqr(X[i]) - X[i + 1]) * P[i] + sqr(X[i] + (-1.0)) * Q[i], hi=n - 1)
    first = lambda j: (X[j] + (-1.0)) * Q2[j] + ((sqr(X[j]) - X[j + 1]) * X[j]) * P4[j]
    mid = lambda j: (((sqr(X[j]) - X[j + 1]) * P4[j] + (Q2[j] + P2[j - 1])) * X[j] + M2Q[j]) - sqr(X[j - 1]) * P2[j - 1]
    last = lambda j: (X[j] - sqr(X[j - 1])) * P2[j - 1]
    secs = [Section(first, 0, 1)]
    if n > 2:
        secs.append(Section(mid, 1, n - 1))
    secs.append(Section(last, n - 1, n))
    return f, Gradient(secs)


def expsqrt(n: int, coef: np.ndarray):
    A, B = float(coef[0]), float(coef[1])
    k = (2 * math.pi) * coef[2:2 + n]
    K = Coef(k)
    inv_n = Const(_rd(Fraction(1) / n), _ru(Fraction(1) / n))
    ape = Const(_rd(Fraction(A) + Fraction(E_LO)), _ru(Fraction(A) + Fraction(E_HI)))
    abn = Const(_rd(Fraction(_rd(Fraction(A) * Fraction(B))) / n), _ru(Fraction(_ru(Fraction(A) * Fraction(B))) / n))
    KN = Coef([_rd(Fraction(v) / n) for v in k], [_ru(Fraction(v) / n) for v in k])
    s = Sum(lambda i: sqr(X[i]))
    cs = Sum(lambda i: cos(X[i] * K[i]))
    r = sqrt(s * inv_n)
    u = exp(cs * inv_n)
    f = (exp(r * (-B)) * (-A) - u) + ape
    gg = (exp(r * (-B)) / r) * abn
    g = lambda j: gg * X[j] + (sin(X[j] * K[j]) * u) * KN[j]
    return f, Gradient(g, skip_if_contains=0.0)


def prodcos(n: int, coef: np.ndarray):
    d = float(coef[0])
    idx = np.arange(1, n + 1, dtype=np.float64)
    RSQ = Coef([_rd(Fraction(1) / Fraction(_sqrt_ru(v))) for v in idx],
               [_ru(Fraction(1) / Fraction(_sqrt_rd(v))) for v in idx])
    inv_d = (_rd(Fraction(1) / Fraction(d)), _ru(Fraction(1) / Fraction(d)))
    INV_D = Const(*inv_d)
    INV_D2 = Const(2.0 * inv_d[0], 2.0 * inv_d[1])
    f = (Sum(lambda i: sqr(X[i])) * INV_D + 1.0) + Prod(lambda i: cos(X[i] * RSQ[i]), init=-1.0)
    P = Prod(lambda i: cos(X[i] * RSQ[i]), init=1.0)

    def g(j):
        a = X[j] * RSQ[j]
        return ((P / cos(a)) * sin(a)) * RSQ[j] + X[j] * INV_D2

    return f, Gradient(g)


BUILTIN = {1: cosquad, 2: chained, 3: expsqrt, 4: prodcos}


# ---------------------------------------------------------------------------
# problems
# ---------------------------------------------------------------------------
def problem(name: str, n: int, tol: float = 1e-6, split: tuple[int, int] | None = None, samples: int = 10,
            domain: tuple[float, float] | None = None, with_gradient: bool | str = True) -> Problem:
    """One of the reference benchmarks as a CODELIST problem of dimension n
    (``with_gradient``: True the restated derivative list, "auto" the derived
    one, False none)."""
    from .problems import default_split
    f, grad, dom = REFERENCE[name](n)
    dom = domain or dom
    g = grad if with_gradient is True else ("auto" if with_gradient == "auto" else None)
    coef = compile_objective(f, n, g).coef
    wid, group = split or default_split(n)
    return Problem(CODELIST, n, np.tile(np.array(dom, dtype=np.float64), n), coef, wid=wid, group=group,
                   samples=samples, stop_mode=STOP_GAP, gap_tol=tol, tag=f"{name}{n}")


def as_codelist(p: Problem) -> Problem:
    """The same problem with its built-in family restated as a code list."""
    import dataclasses
    f, grad = BUILTIN[p.family](p.n, p.coef)
    coef = compile_objective(f, p.n, grad).coef
    return dataclasses.replace(p, family=CODELIST, coef=coef, tag=p.tag + "-cl")
