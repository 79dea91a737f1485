"""Problem descriptions and seeded synthetic instances.

A :class:`Problem` is the per-problem input of the reference scripts made
explicit: objective family and coefficients (the reference hard-codes them in
each code list, e.g. GPUGO_1.1/7-Rastrigin/rastrigin50.py:161-188), box domain
(``initialRegion``, rastrigin50.py:852), split rule (``wid`` parts over a cycled
group of ``group`` coordinates, rastrigin50.py:420-423), sample count
(``numSamples``, :909), stopping rule (``widthTolerance``, :904) and initial
upper bound (``lowestUpperVal``, :888).

Families (coefficient layout in ``coef``):

* ``COSQUAD``  f = sum_i a_i x_i^2 - b_i cos(K_i x_i) + sum_i b_i,
  K_i = fl(fl(2 pi) c_i)                                       coef = a[n], b[n], c[n]
* ``CHAINED``  f = sum_{i<n} p_i (x_{i+1} - x_i^2)^2 + q_i (1 - x_i)^2   coef = p[n-1], q[n-1]
* ``EXPSQRT``  f = -A exp(-B sqrt(mean x^2)) - exp(mean cos(K_i x_i)) + A + e,
  K_i = fl(fl(2 pi) w_i)                                       coef = A, B, w[n]
* ``PRODCOS``  f = 1 + sum_i x_i^2 / d - prod_i cos(x_i / sqrt(i))      coef = d
* ``CODELIST`` any objective compiled by :mod:`gpugo_gb300.codelist`   coef = the code list

The reference's Rastrigin, Rosenbrock, Ackley and Griewank scripts are the
special cases a=1,b=10,c=1 / p=100,q=1 / A=20,B=0.02,w=1 / d=4000.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

COSQUAD, CHAINED, EXPSQRT, PRODCOS, CODELIST = 1, 2, 3, 4, 5
FAMILY_NAMES = {COSQUAD: "cosquad", CHAINED: "chained", EXPSQRT: "expsqrt", PRODCOS: "prodcos", CODELIST: "codelist"}
STOP_WIDTH, STOP_GAP = 0, 1
MASTER_SEED = 0x6770756F


@dataclass
class Problem:
    family: int
    n: int
    domain: np.ndarray            # [2n]: lo_1, hi_1, ..., lo_n, hi_n
    coef: np.ndarray
    wid: int = 4
    group: int = 10
    samples: int = 10
    stop_mode: int = STOP_GAP
    width_tol: float = 0.0
    gap_tol: float = 1e-6
    ub_init: float = math.inf
    max_iter: int = 0             # 0: unlimited
    pool_cap: int = 0             # 0: chosen by the engine
    parent_cap: int = 0           # 0: chosen by the engine
    tag: str = field(default="", compare=False)

    def __post_init__(self):
        self.domain = np.ascontiguousarray(self.domain, dtype=np.float64).ravel()
        self.coef = np.ascontiguousarray(self.coef, dtype=np.float64).ravel()
        if self.domain.size != 2 * self.n:
            raise ValueError("domain must hold 2n bounds")

    @property
    def children_per_iter(self) -> int:
        return self.wid ** min(self.group, self.n)

    def evaluate(self, x: np.ndarray) -> float:
        """Plain FP64 point evaluation (no rounding control), for checks."""
        x = np.asarray(x, dtype=np.float64)
        n = self.n
        c = self.coef
        if self.family == COSQUAD:
            a, b, cc = c[:n], c[n:2 * n], c[2 * n:3 * n]
            k = (2 * math.pi) * cc
            return float(np.sum(a * x * x - b * np.cos(k * x)) + np.sum(b))
        if self.family == CHAINED:
            p, q = c[:n - 1], c[n - 1:2 * n - 2]
            return float(np.sum(p * (x[1:] - x[:-1] ** 2) ** 2 + q * (1 - x[:-1]) ** 2))
        if self.family == EXPSQRT:
            A, B, w = c[0], c[1], c[2:2 + n]
            k = (2 * math.pi) * w
            return float(-A * math.exp(-B * math.sqrt(np.mean(x * x))) - math.exp(np.mean(np.cos(k * x)))
                         + A + math.e)
        if self.family == PRODCOS:
            d = c[0]
            i = np.arange(1, n + 1, dtype=np.float64)
            return float(1 + np.sum(x * x) / d - np.prod(np.cos(x / np.sqrt(i))))
        if self.family == CODELIST:
            from .codelist import point_value
            return point_value(self.coef, x)
        raise ValueError(self.family)

    def minimiser(self) -> np.ndarray:
        return np.ones(self.n) if self.family == CHAINED else np.zeros(self.n)


def default_split(n: int) -> tuple[int, int]:
    """Split rule (wid, group) for generated instances: an odd number of parts,
    so that a minimiser at the centre of a symmetric domain lies inside one child
    instead of on the shared corner of all of them (where every child has the same
    LB and the reference's first-in-list tie-break expands them breadth first),
    with 700-16K children per iteration and cycles of 8 coordinates above n = 8."""
    table = {1: (63, 1), 2: (31, 2), 3: (9, 3), 4: (7, 4), 5: (5, 5), 6: (5, 6), 7: (3, 7)}
    if n in table:
        return table[n]
    return (3, 8)


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def cosquad(n: int, rng: np.random.Generator, lo=-5.12, hi=5.12) -> tuple[np.ndarray, np.ndarray]:
    a = rng.uniform(0.5, 2.0, n)
    b = rng.uniform(5.0, 15.0, n)
    c = rng.integers(1, 3, n).astype(np.float64)
    return np.tile([lo, hi], n), np.concatenate([a, b, c])


def chained(n: int, rng: np.random.Generator, lo=-5.0, hi=10.0):
    p = rng.uniform(50.0, 150.0, n - 1)
    q = rng.uniform(0.5, 2.0, n - 1)
    return np.tile([lo, hi], n), np.concatenate([p, q])


def expsqrt(n: int, rng: np.random.Generator, lo=-32.768, hi=32.768):
    A = rng.uniform(15.0, 25.0)
    B = rng.uniform(0.1, 0.3)
    w = rng.uniform(0.8, 1.2, n)
    return np.tile([lo, hi], n), np.concatenate([[A, B], w])


def prodcos(n: int, rng: np.random.Generator, lo=-600.0, hi=600.0):
    d = rng.uniform(2000.0, 6000.0)
    return np.tile([lo, hi], n), np.array([d])


_GEN = {COSQUAD: cosquad, CHAINED: chained, EXPSQRT: expsqrt, PRODCOS: prodcos}


def instance(family: int, n: int, seed: int, tol: float = 1e-6, split: tuple[int, int] | None = None,
             samples: int = 10, tag: str = "") -> Problem:
    rng = _rng(seed)
    if family == CHAINED and n < 2:
        n = 2
    dom, coef = _GEN[family](n, rng)
    wid, group = split or default_split(n)
    return Problem(family, n, dom, coef, wid=wid, group=group, samples=samples, stop_mode=STOP_GAP,
                   gap_tol=tol, tag=tag or f"{FAMILY_NAMES[family]}{n}")


def config1(seed: int = MASTER_SEED + 1) -> Problem:
    """n=2 cosine-quadratic on [-5.12,5.12]^2, 64x64 grid, UB-LB <= 1e-6."""
    return instance(COSQUAD, 2, seed, 1e-6, (64, 2), tag="cfg1-cosquad2")


def config2(seed: int = MASTER_SEED + 2) -> Problem:
    """n=8 chained quartic on [-5,10]^8, 4^8 grid, UB-LB <= 1e-6."""
    return instance(CHAINED, 8, seed, 1e-6, (4, 8), tag="cfg2-chained8")


def config3(seed: int = MASTER_SEED + 3, split: tuple[int, int] = (2, 32)) -> Problem:
    """n=32 exp-sqrt composite on [-32.768,32.768]^32, 2^32-cell split, UB-LB <= 1e-4."""
    return instance(EXPSQRT, 32, seed, 1e-4, split, tag="cfg3-expsqrt32")


def _log_uniform_n(rng: np.random.Generator, lo: int, hi: int) -> int:
    return int(min(hi, max(lo, round(math.exp(rng.uniform(math.log(lo), math.log(hi + 0.5)))))))


def config4(count: int = 1024, seed: int = MASTER_SEED + 4, nmax: int = 64) -> list[Problem]:
    """Mixed batch: families F1-F4, n log-uniform in {2..nmax}, UB-LB <= 1e-6."""
    rng = _rng(seed)
    out = []
    for i in range(count):
        fam = int(rng.integers(1, 5))
        n = _log_uniform_n(rng, 2, nmax)
        out.append(instance(fam, n, int(rng.integers(0, 2 ** 63)), 1e-6, tag=f"b{i}"))
    return out


def config5(count: int = 4096, seed: int = MASTER_SEED + 5, nmax: int = 128, rate: float = 0.0):
    """Serving stream: (arrival time, Problem) pairs with Poisson arrivals."""
    rng = _rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        fam = int(rng.integers(1, 5))
        n = _log_uniform_n(rng, 2, nmax)
        tol = 1e-6 if rng.random() < 0.5 else 1e-4
        if rate > 0:
            t += float(rng.exponential(1.0 / rate))
        out.append((t, instance(fam, n, int(rng.integers(0, 2 ** 63)), tol, tag=f"r{i}")))
    return out
