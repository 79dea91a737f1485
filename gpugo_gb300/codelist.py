"""Objective front end: expressions -> code lists for the CODELIST family.

The reference writes each objective as three hand-made code lists of interval
operations: value (e.g. GPUGO_1.1/6-Levy/levy50.py:141-226), sample (:235-379,
the value list run on the points of the box diagonal) and derivative (:382-563,
one gradient component per coordinate followed by the generalized KKT test).
This module builds the same kind of list from an expression written with
Python operators, so that objectives beyond the four built-in families run on
the device without new kernels:

    from gpugo_gb300.codelist import X, Sum, sin, sqr, compile_objective
    f = Sum(lambda i: sqr(X[i]) * 0.5 - sin(X[i] * 3.0))
    coef = compile_objective(f, n=16, gradient=Gradient(lambda j: X[j] - cos(X[j] * 3.0) * 3.0))

Every operator maps to one operation of the reference's interval library
(Updated Interval Arithmetic Operations/IA.py): ``e + e`` add, ``e - e`` minus,
``e * e`` multiply, ``e / e`` divide, ``e * c`` times (scalar), ``e + c`` plus
(scalar), ``e ** 2`` power 2, ``e ** 0.5`` power 0.5, and ``sin``, ``cos``,
``exp``.  The grouping written is the grouping evaluated: ``(a + b) + c`` and
``a + (b + c)`` are different code lists, as they are in the reference.
``Sum`` and ``Prod`` run the reference's accumulation loops (start value, then
``acc = add(acc, term)`` / ``acc = multiply(acc, term)`` for i = lo .. hi-1).

Format of the compiled coefficient array (``gpugo_spec.coef`` of family
``GPUGO_CODELIST``).  Word k of the header and of the code is stored in the low
32 bits of coef[k] (the high 32 bits are zero), so the array holds only finite
values and every copy keeps it bit for bit:

    [0] 0x314C4347  [1] n  [2] registers  [3] instructions  [4] constants
    [5] value start [6] value length  [7] gradient prologue start [8] length
    [9] sections    [10] skip constant (0xFFFFFFFF: none)  [11] value result register
    [12] term tables  [13..15] 0
    [16 + 12s ...]  section s: lo, hi, start, length, gradient register, check
                    offset, skip register (0xFFFFFFFF: none; the test is skipped
                    when that register has an infinite end), tabled (0/1),
                    offsets (0..3), offset 0, offset 1, offset 2
    [U + 12t ...]   term table t: lo, hi, kind (0 sum, 1 product), offsets (0..2),
                    offset 0, offset 1, 0, body start, body length, body result
                    register, 0, 0
    [I + 4t ...]    instruction t: op | dst << 8 | a << 16 | b << 24, imm1, imm2, 0
    [C ...]         constants (plain doubles)

with U = 16 + 12 sections, I = U + 12 tables and C = I + 4 instructions.

Term tables.  A Sum or Prod whose body reads the coordinates only as X[i + o]
(at most two offsets o) and otherwise only coefficients and constants is a
*table reduction* (instruction TRED): the body is a separate piece of code with
its own registers, and the device evaluates it once per iteration for every
coordinate i, every digit of the coordinates i + o and every sample pass into a
table; a child then adds (multiplies) its entries.  The result is the one the
loop gives: the same operations on the same inputs, accumulated in the same
order.  Other bodies run as a loop (LOOP .. ENDLOOP) in the child's code.

Tabled sections.  A gradient section whose expression reads the coordinates only
as X[j + o] (at most three offsets, the KKT test's own coordinate included) and
otherwise constants and coefficients is compiled self-contained (it reads no
prologue register); the device evaluates its KKT test once per iteration for
every coordinate j and digit combination of the coordinates j + o, and a
candidate only looks its flags up.  The flag is the one the section's code gives.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np

MAGIC = 0x314C4347
MAX_REGS = 16
HEADER = 16
SEC_WORDS = 12
MAX_TABLED_SECTIONS = 8
MAX_SECTION_OFFSETS = 3
TAB_WORDS = 12
INS_WORDS = 4
MAX_TABLES = 8
MAX_TABLE_OFFSETS = 2
NO_SKIP = 0xFFFFFFFF

# opcodes (the device interpreter and the oracle use the same numbers)
LDX, LDC, LDI, LDK, LDKI, ADD, MINUS, MUL, DIV, TIMES, PLUS, TIMESK, PLUSK, SQR, SQRT, EXP, SIN, COS, MOV, \
    LOOP, ENDLOOP, TRED = range(1, 23)
OP_NAMES = {v: k for k, v in dict(
    LDX=LDX, LDC=LDC, LDI=LDI, LDK=LDK, LDKI=LDKI, ADD=ADD, MINUS=MINUS, MUL=MUL, DIV=DIV, TIMES=TIMES, PLUS=PLUS,
    TIMESK=TIMESK, PLUSK=PLUSK, SQR=SQR, SQRT=SQRT, EXP=EXP, SIN=SIN, COS=COS, MOV=MOV, LOOP=LOOP,
    ENDLOOP=ENDLOOP, TRED=TRED).items()}
# index bases of LDX / LDK / LDKI / TIMESK / PLUSK
BASE_ABS, BASE_I, BASE_J = 0, 1, 2
NO_REG = 0xFFFFFFFF


class CodeListError(ValueError):
    pass


# ---------------------------------------------------------------------------
# index expressions: the loop index i of Sum/Prod and the gradient coordinate j
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Index:
    base: int          # BASE_I or BASE_J
    off: int = 0

    def __add__(self, k: int) -> "Index":
        return Index(self.base, self.off + int(k))

    __radd__ = __add__

    def __sub__(self, k: int) -> "Index":
        return Index(self.base, self.off - int(k))


def _index(k) -> tuple[int, int]:
    if isinstance(k, Index):
        return k.base, k.off
    if isinstance(k, (int, np.integer)):
        return BASE_ABS, int(k)      # negative: from the end, resolved with n
    raise CodeListError(f"bad coordinate index {k!r}")


# ---------------------------------------------------------------------------
# expression nodes
# ---------------------------------------------------------------------------
class Expr:
    __slots__ = ("op", "args", "key")

    def __init__(self, op: str, args: tuple):
        self.op = op
        self.args = args
        self.key = (op,) + tuple(a.key if isinstance(a, Expr) else a for a in args)

    # arithmetic: scalars become the reference's scalar operations (times/plus)
    def __add__(self, o):
        if _scalar(o):
            return Expr("plus", (self, _f(o)))
        if isinstance(o, CoefRef) and o.op == "ldk" and not isinstance(self, CoefRef):
            return Expr("plusk", (self, o))
        return Expr("add", (self, _e(o)))

    def __radd__(self, o):
        return self.__add__(o)

    def __sub__(self, o):
        if _scalar(o):
            return Expr("plus", (self, -_f(o)))
        return Expr("minus", (self, _e(o)))

    def __rsub__(self, o):
        return Expr("minus", (_e(o), self))

    def __mul__(self, o):
        if _scalar(o):
            return Expr("times", (self, _f(o)))
        if isinstance(o, CoefRef) and o.op == "ldk" and not isinstance(self, CoefRef):
            return Expr("timesk", (self, o))
        return Expr("mul", (self, _e(o)))

    def __rmul__(self, o):
        return self.__mul__(o)

    def __truediv__(self, o):
        return Expr("div", (self, _e(o)))

    def __rtruediv__(self, o):
        return Expr("div", (_e(o), self))

    def __neg__(self):
        return Expr("times", (self, -1.0))

    def __pow__(self, p):
        if p == 2:
            return Expr("sqr", (self,))
        if p == 0.5:
            return Expr("sqrt", (self,))
        raise CodeListError("only the powers 2 and 0.5 of the interval library are available")

    def __repr__(self):
        return f"Expr{self.key}"


def _scalar(o) -> bool:
    return isinstance(o, (int, float, np.floating, np.integer)) and not isinstance(o, bool)


def _f(o) -> float:
    return float(o)


def _e(o) -> Expr:
    if isinstance(o, Expr):
        return o
    if _scalar(o):
        return Const(float(o))
    raise CodeListError(f"cannot use {o!r} in an expression")


class CoefRef(Expr):
    """Element of a per-coordinate coefficient array: a point interval, or an
    interval for arrays made with :func:`coef_interval`.  ``K[i] * e`` and
    ``K[i] + e`` are the scalar operations times/plus, as ``e * K[i]``."""
    __slots__ = ()

    def __mul__(self, o):
        if self.op == "ldk" and isinstance(o, Expr) and not isinstance(o, CoefRef):
            return Expr("timesk", (o, self))
        return Expr.__mul__(self, o)

    def __add__(self, o):
        if self.op == "ldk" and isinstance(o, Expr) and not isinstance(o, CoefRef):
            return Expr("plusk", (o, self))
        return Expr.__add__(self, o)


def Const(lo: float, hi: float | None = None) -> Expr:
    """A constant: the point interval [lo, lo], or [lo, hi]."""
    lo = float(lo)
    if hi is None:
        return Expr("ldc", (_bits(lo),))
    hi = float(hi)
    if not lo <= hi:
        raise CodeListError("interval constant with lo > hi")
    return Expr("ldi", (_bits(lo), _bits(hi)))


def _bits(v: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", v))[0]


class _XIndexer:
    def __getitem__(self, k) -> Expr:
        base, off = _index(k)
        return Expr("x", (base, off))


X = _XIndexer()
"""Coordinate intervals: ``X[i]``, ``X[i + 1]`` (loop index), ``X[j]``
(gradient coordinate), ``X[0]``, ``X[-1]`` (fixed coordinates)."""


class Coef:
    """A per-coordinate coefficient array (``len(values)`` entries)."""

    def __init__(self, values, hi=None):
        lo = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self.interval = hi is not None
        if self.interval:
            hi = np.ascontiguousarray(hi, dtype=np.float64).ravel()
            if hi.shape != lo.shape or not np.all(lo <= hi):
                raise CodeListError("interval coefficients need lo <= hi of the same length")
            self.data = np.stack([lo, hi], axis=1).ravel()
        else:
            self.data = lo
        self.length = lo.size
        self.key_bits = tuple(_bits(v) for v in self.data)

    def __getitem__(self, k) -> CoefRef:
        base, off = _index(k)
        r = CoefRef.__new__(CoefRef)
        Expr.__init__(r, "ldki" if self.interval else "ldk", (base, off, self))
        return r

    # identity of an array inside keys
    def __hash__(self):
        return hash(self.key_bits)

    def __eq__(self, o):
        return isinstance(o, Coef) and o.interval == self.interval and o.key_bits == self.key_bits

    def __repr__(self):
        return f"Coef(len={self.length}, interval={self.interval})"


def coef_interval(lo, hi) -> Coef:
    return Coef(lo, hi)


def sin(e) -> Expr:
    return Expr("sin", (_e(e),))


def cos(e) -> Expr:
    return Expr("cos", (_e(e),))


def exp(e) -> Expr:
    return Expr("exp", (_e(e),))


def sqrt(e) -> Expr:
    return Expr("sqrt", (_e(e),))


def sqr(e) -> Expr:
    return Expr("sqr", (_e(e),))


_I = Index(BASE_I)
_J = Index(BASE_J)


def _reduce(kind: str, body: Callable[[Index], Expr], lo: int, hi: int | None, init) -> Expr:
    b = body(_I)
    if _scalar(b):
        b = Const(float(b))
    if not isinstance(b, Expr):
        raise CodeListError("a Sum/Prod body must return an expression")
    init_e = _e(init)
    return Expr(kind, (b, int(lo), None if hi is None else int(hi), init_e))


def Sum(body: Callable[[Index], Expr], lo: int = 0, hi: int | None = None, init=0.0) -> Expr:
    """init + term(lo) + ... + term(hi-1), accumulated left to right with the
    interval add (hi None: n; negative: n + hi)."""
    return _reduce("sum", body, lo, hi, init)


def Prod(body: Callable[[Index], Expr], lo: int = 0, hi: int | None = None, init=1.0) -> Expr:
    """init * term(lo) * ... * term(hi-1) with the interval multiply."""
    return _reduce("prod", body, lo, hi, init)


@dataclass
class Section:
    """Gradient component for coordinates j in [lo, hi): ``expr(j)``; the KKT
    test reads the bounds of coordinate j + check (0 in a correct code list).
    ``skip_infinite(j)`` (optional) names a sub-expression: when it has an
    infinite end the coordinate is not tested (corrupted50.py:418-421)."""
    expr: Callable[[Index], Expr]
    lo: int = 0
    hi: int | None = None
    check: int = 0
    skip_infinite: Callable[[Index], Expr] | None = None


@dataclass
class Gradient:
    """Derivative code list: one or more sections covering the coordinates, and
    optionally the reference's skip rule for boxes that contain a given point in
    every coordinate (ackley50.py:402-409, salomon50.py's origin test)."""
    sections: list[Section] | Callable[[Index], Expr]
    skip_if_contains: float | None = None

    def __post_init__(self):
        if callable(self.sections) and not isinstance(self.sections, list):
            self.sections = [Section(self.sections)]


# ---------------------------------------------------------------------------
# automatic gradient
# ---------------------------------------------------------------------------
_ONE = None   # set below (Const(1.0)); None stands for an exact zero


def _is_one(e) -> bool:
    return e is not None and e.key == _ONE.key


def _add(u, v):
    if u is None:
        return v
    if v is None:
        return u
    return Expr("add", (u, v))


def _sub(u, v):
    if v is None:
        return u
    if u is None:
        return Expr("times", (v, -1.0))
    return Expr("minus", (u, v))


def _mul(u, v):
    if u is None or v is None:
        return None
    if _is_one(u):
        return v
    if _is_one(v):
        return u
    return Expr("mul", (u, v))


def _times(u, c: float):
    if u is None:
        return None
    if _is_one(u):
        return Const(c)
    return Expr("times", (u, c))


def _diff(e: Expr, wrt_key, memo: dict):
    """d e / d (the node with key wrt_key), None for an exact zero.  Reductions
    and coordinates other than wrt are constants here."""
    k = e.key
    if k == wrt_key:
        return _ONE
    if k in memo:
        return memo[k]
    op, a = e.op, e.args
    if op in ("x", "ldc", "ldi", "ldk", "ldki", "sum", "prod"):
        r = None
    elif op in ("add", "minus"):
        da, db = _diff(a[0], wrt_key, memo), _diff(a[1], wrt_key, memo)
        r = _add(da, db) if op == "add" else _sub(da, db)
    elif op == "mul":
        r = _add(_mul(_diff(a[0], wrt_key, memo), a[1]), _mul(a[0], _diff(a[1], wrt_key, memo)))
    elif op == "div":
        da, db = _diff(a[0], wrt_key, memo), _diff(a[1], wrt_key, memo)
        # (da - (a / b) db) / b
        num = _sub(da, _mul(e, db))
        r = None if num is None else Expr("div", (num, a[1]))
    elif op == "times":
        r = _times(_diff(a[0], wrt_key, memo), a[1])
    elif op == "plus" or op == "plusk":
        r = _diff(a[0], wrt_key, memo)
    elif op == "timesk":
        da = _diff(a[0], wrt_key, memo)
        r = None if da is None else (a[1] if _is_one(da) else Expr("timesk", (da, a[1])))
    elif op == "sqr":
        r = _times(_mul(a[0], _diff(a[0], wrt_key, memo)), 2.0)
    elif op == "sqrt":
        da = _diff(a[0], wrt_key, memo)
        r = None if da is None else _times(Expr("div", (da, e)), 0.5)
    elif op == "exp":
        r = _mul(e, _diff(a[0], wrt_key, memo))
    elif op == "sin":
        r = _mul(Expr("cos", (a[0],)), _diff(a[0], wrt_key, memo))
    elif op == "cos":
        r = _times(_mul(Expr("sin", (a[0],)), _diff(a[0], wrt_key, memo)), -1.0)
    else:
        raise CodeListError(f"no derivative rule for {op}")
    memo[k] = r
    return r


def _leaves(e: Expr, out: dict):
    """Reductions and fixed coordinates of the value expression (outside bodies)."""
    if not isinstance(e, Expr):
        return
    if e.op in ("sum", "prod"):
        out[e.key] = e
        return
    if e.op == "x":
        if e.args[0] != BASE_ABS:
            raise CodeListError("the value expression reads X[i] outside a Sum/Prod")
        out[e.key] = e
        return
    for a in e.args:
        if isinstance(a, Expr):
            _leaves(a, out)


def _shift(e, o: int, memo: dict):
    """The body expression with the loop index i replaced by j - o (memo is per o)."""
    if not isinstance(e, Expr):
        return e
    if e.key in memo:
        return memo[e.key]
    if e.op == "x":
        base, off = e.args
        r = Expr("x", (BASE_J, off - o)) if base == BASE_I else e
    elif e.op in ("ldk", "ldki"):
        base, off, arr = e.args
        r = arr[Index(BASE_J, off - o)] if base == BASE_I else e
    elif e.op in ("sum", "prod"):
        r = e   # an inner reduction binds its own loop index
    else:
        args = tuple(_shift(a, o, memo) for a in e.args)
        r = CoefRef.__new__(CoefRef) if isinstance(e, CoefRef) else Expr.__new__(Expr)
        Expr.__init__(r, e.op, args)
    memo[e.key] = r
    return r


def _rebase_abs(e, c: int, n: int, memo: dict):
    """In a section of the single coordinate c, the fixed coordinate X[k] is X[j + k - c]."""
    if not isinstance(e, Expr):
        return e
    if e.key in memo:
        return memo[e.key]
    if e.op == "x" and e.args[0] == BASE_ABS:
        k = e.args[1] + n if e.args[1] < 0 else e.args[1]
        r = Expr("x", (BASE_J, k - c))
    elif e.op in ("x", "ldc", "ldi", "ldk", "ldki", "sum", "prod"):
        r = e
    else:
        args = tuple(_rebase_abs(a, c, n, memo) for a in e.args)
        r = CoefRef.__new__(CoefRef) if isinstance(e, CoefRef) else Expr.__new__(Expr)
        Expr.__init__(r, e.op, args)
    memo[e.key] = r
    return r


def _body_leaves(e, out: dict):
    """Fixed coordinates and (loop-invariant) reductions inside a reduction's body."""
    if not isinstance(e, Expr):
        return
    if e.op in ("sum", "prod") or (e.op == "x" and e.args[0] == BASE_ABS):
        out[e.key] = e
        return
    for a in e.args:
        if isinstance(a, Expr):
            _body_leaves(a, out)


def _xi_offsets(e, acc: set):
    """Offsets o of the X[i + o] a body reads (outside its inner reductions)."""
    if not isinstance(e, Expr) or e.op in ("sum", "prod"):
        return
    if e.op == "x":
        if e.args[0] == BASE_I:
            acc.add(e.args[1])
        elif e.args[0] == BASE_J:
            raise CodeListError("the value expression reads the gradient coordinate j")
        return
    for a in e.args:
        if isinstance(a, Expr):
            _xi_offsets(a, acc)


def auto_gradient(f: Expr, n: int) -> Gradient:
    """The gradient code list of a value expression, by symbolic differentiation.

    d f / d x_j = sum over reductions R of (d f / d R) (d R / d x_j) plus, for a
    fixed coordinate X[k], d f / d X[k] when j = k.  For R = Sum_i t(i):
    d R / d x_j = sum over the offsets o of t of (d t / d X[i+o]) at i = j - o,
    for j - o in R's range; for a product, (R / t(j - o)) (d t / d X[i+o]).
    A fixed coordinate or another reduction L inside t is reached through R with
    d R / d L = Sum_i d t(i) / d L (for a product Sum_i (R / t(i)) d t(i) / d L),
    a reduction over R's range evaluated once per box; such leaves go through a
    worklist with their accumulated adjoints.  The coordinates where the set of
    terms changes split [0, n) into sections.  Every rule is exact, so the
    interval evaluation encloses the gradient; a division by an interval
    containing zero (a product's term, a square root at zero) gives an unbounded
    gradient and the test keeps the box."""
    global _ONE
    if _ONE is None:
        _ONE = Const(1.0)
    leaves: dict = {}
    _leaves(f, leaves)
    # worklist of (leaf, adjoint); the adjoints of a leaf reached along several
    # paths add up (every path's term is kept: the sum of the exact terms)
    work = [(L, _diff(f, k, {})) for k, L in leaves.items()]
    parts = []
    steps = 0
    while work:
        L, adj = work.pop(0)
        steps += 1
        if steps > 10000:
            raise CodeListError("automatic gradient: the expression is too deeply nested")
        if adj is None:
            continue
        if L.op == "x":
            c = L.args[1] + n if L.args[1] < 0 else L.args[1]
            if not 0 <= c < n:
                raise CodeListError(f"coordinate {L.args[1]} outside 0..{n - 1}")
            parts.append((c, c + 1, adj))
            continue
        body, lo, hi, init = L.args
        hi = n if hi is None else (hi + n if hi < 0 else hi)
        lo = lo + n if lo < 0 else lo
        if lo >= hi:
            continue
        # a start value that reads the coordinates: d R / d init is 1 for a sum,
        # R / init for a product
        init_leaves: dict = {}
        if isinstance(init, Expr):
            _leaves(init, init_leaves)
        for k2, L2 in init_leaves.items():
            d_init = _diff(init, k2, {})
            if L.op == "prod":
                d_init = _mul(Expr("div", (L, init)), d_init)
            work.append((L2, _mul(adj, d_init)))
        offs: set = set()
        _xi_offsets(body, offs)
        for o in sorted(offs):
            dt = _diff(body, Expr("x", (BASE_I, o)).key, {})
            if dt is None:
                continue
            memo: dict = {}
            dj = _shift(dt, o, memo)
            if L.op == "prod":
                dj = _mul(Expr("div", (L, _shift(body, o, memo))), dj)
            parts.append((lo + o, hi + o, _mul(adj, dj)))
        inner: dict = {}
        _body_leaves(body, inner)
        for k2, L2 in inner.items():
            dt = _diff(body, k2, {})
            if dt is None:
                continue
            term = dt if L.op == "sum" else _mul(Expr("div", (L, body)), dt)
            red = Expr("sum", (term, lo, hi, Const(0.0)))
            work.append((L2, _mul(adj, red)))
    cuts = sorted({0, n} | {max(0, min(n, p[0])) for p in parts} | {max(0, min(n, p[1])) for p in parts})
    sections = []
    for a, b in zip(cuts[:-1], cuts[1:]):
        if a >= b:
            continue
        terms = [e for lo, hi, e in parts if lo <= a and b <= hi]
        if not terms:
            continue
        g = terms[0]
        for t in terms[1:]:
            g = Expr("add", (g, t))
        if b - a == 1:
            g = _rebase_abs(g, a, n, {})   # lets the section read its coordinates as X[j + o] (tabled)
        sections.append(Section(lambda j, g=g: g, a, b))
    return Gradient(sections)


# ---------------------------------------------------------------------------
# compiler
# ---------------------------------------------------------------------------
@dataclass
class _Ins:
    op: int
    dst: int = 0        # value id before register allocation
    a: int = 0
    b: int = 0
    imm1: int = 0
    imm2: int = 0
    reads: tuple = ()
    writes: int = -1    # value id


@dataclass
class _Ctx:
    n: int
    consts: list = field(default_factory=list)
    const_ix: dict = field(default_factory=dict)
    arrays: dict = field(default_factory=dict)
    ins: list = field(default_factory=list)
    nval: int = 0
    tables: list = field(default_factory=list)
    table_ix: dict = field(default_factory=dict)
    use_tables: bool = True

    def table(self, kind: int, lo: int, hi: int, offs: list, body: "Expr") -> int:
        """Index of the term table of this reduction (compiled on first use)."""
        key = (kind, lo, hi, body.key)
        if key in self.table_ix:
            return self.table_ix[key]
        sub = _Ctx(self.n)
        sub.consts, sub.const_ix, sub.arrays = self.consts, self.const_ix, self.arrays
        em = _Emitter(sub)
        r = em.emit(body, (lo, hi))
        nreg, reg = _allocate(sub.ins, {r: len(sub.ins) - 1})
        self.tables.append(dict(kind=kind, lo=lo, hi=hi, offs=offs, ins=sub.ins, reg=reg[r], nreg=nreg))
        self.table_ix[key] = len(self.tables) - 1
        return self.table_ix[key]

    def const(self, bits: int) -> int:
        if bits not in self.const_ix:
            self.const_ix[bits] = len(self.consts)
            self.consts.append(bits)
        return self.const_ix[bits]

    def const_pair(self, lo_bits: int, hi_bits: int) -> int:
        # an interval constant occupies two consecutive slots
        for k in range(len(self.consts) - 1):
            if self.consts[k] == lo_bits and self.consts[k + 1] == hi_bits:
                return k
        k = len(self.consts)
        self.consts += [lo_bits, hi_bits]
        return k

    def array(self, arr: Coef) -> int:
        if arr not in self.arrays:
            self.arrays[arr] = len(self.consts)
            self.consts += list(arr.key_bits)
        return self.arrays[arr]

    def new_val(self) -> int:
        self.nval += 1
        return self.nval - 1


def _section_offsets(e, acc: set) -> bool:
    """True when a gradient section reads coordinates only as X[j + o]
    (collected in acc) and contains no reduction."""
    if not isinstance(e, Expr):
        return True
    if e.op == "x":
        if e.args[0] != BASE_J:
            return False
        acc.add(e.args[1])
        return True
    if e.op in ("ldk", "ldki"):
        return e.args[0] != BASE_I
    if e.op in ("sum", "prod"):
        return False
    return all(_section_offsets(a, acc) for a in e.args if isinstance(a, Expr))


def _table_offsets(e, acc: set) -> bool:
    """True when the body reads coordinates only as X[i + o] (collected in acc)
    and holds no reduction and nothing of the gradient coordinate."""
    if not isinstance(e, Expr):
        return True
    if e.op == "x":
        if e.args[0] != BASE_I:
            return False
        acc.add(e.args[1])
        return True
    if e.op in ("ldk", "ldki"):
        return e.args[0] != BASE_J
    if e.op in ("sum", "prod"):
        return False
    return all(_table_offsets(a, acc) for a in e.args if isinstance(a, Expr))


def _depends(e, base: int, memo: dict) -> bool:
    """True when the expression reads the index of the given base."""
    if not isinstance(e, Expr):
        return False
    k = (e.key, base)
    if k in memo:
        return memo[k]
    if e.op in ("x", "ldk", "ldki"):
        r = e.args[0] == base
    elif e.op in ("sum", "prod"):
        # the loop index of a reduction is bound inside it
        r = False if base == BASE_I else _depends(e.args[0], base, memo) or _depends(e.args[3], base, memo)
    else:
        r = any(_depends(a, base, memo) for a in e.args if isinstance(a, Expr))
    memo[k] = r
    return r


class _Emitter:
    """Linear code with common subexpressions evaluated once.  Values that do
    not read the loop index are evaluated before the loop that uses them."""

    def __init__(self, ctx: _Ctx, section: int = -1):
        self.ctx = ctx
        self.done: dict = {}       # (key, scope) -> value id
        self.dep: dict = {}
        self.section = section
        self.sec_range = (0, 0)

    def _idx(self, base: int, off: int, lo: int | None = None, hi: int | None = None) -> tuple[int, int]:
        n = self.ctx.n
        if base == BASE_ABS:
            k = off + n if off < 0 else off
            if not 0 <= k < n:
                raise CodeListError(f"coordinate {off} outside 0..{n - 1}")
            return BASE_ABS, k
        return base, off

    def emit(self, e: Expr, scope) -> int:
        """scope: None (straight code) or the loop range (lo, hi) when inside a loop."""
        inside = scope is not None and _depends(e, BASE_I, self.dep)
        key = (e.key, scope if inside else None)
        if key in self.done:
            return self.done[key]
        sc = scope if inside else None
        ctx = self.ctx
        op = e.op
        v = ctx.new_val()
        if op == "x":
            base, off = self._idx(*e.args)
            self._check_range(base, off, sc)
            ctx.ins.append(_Ins(LDX, v, base, 0, off, 0, (), v))
        elif op == "ldc":
            ctx.ins.append(_Ins(LDC, v, 0, 0, 0, ctx.const(e.args[0]), (), v))
        elif op == "ldi":
            ctx.ins.append(_Ins(LDI, v, 0, 0, 0, ctx.const_pair(e.args[0], e.args[1]), (), v))
        elif op in ("ldk", "ldki"):
            base, off, arr = e.args
            base, off = self._idx(base, off)
            self._check_range(base, off, sc, arr.length)
            ctx.ins.append(_Ins(LDK if op == "ldk" else LDKI, v, base, 0, off, ctx.array(arr), (), v))
        elif op in ("add", "minus", "mul", "div"):
            a = self.emit(e.args[0], scope)
            b = self.emit(e.args[1], scope)
            code = {"add": ADD, "minus": MINUS, "mul": MUL, "div": DIV}[op]
            ctx.ins.append(_Ins(code, v, a, b, 0, 0, (a, b), v))
        elif op in ("times", "plus"):
            a = self.emit(e.args[0], scope)
            ctx.ins.append(_Ins(TIMES if op == "times" else PLUS, v, a, 0, 0, ctx.const(_bits(e.args[1])), (a,), v))
        elif op in ("timesk", "plusk"):
            a = self.emit(e.args[0], scope)
            ref = e.args[1]
            if ref.op != "ldk":
                raise CodeListError("scalar times/plus take a point coefficient array")
            base, off, arr = ref.args
            base, off = self._idx(base, off)
            self._check_range(base, off, sc, arr.length)
            ctx.ins.append(_Ins(TIMESK if op == "timesk" else PLUSK, v, a, base, off, ctx.array(arr), (a,), v))
        elif op in ("sqr", "sqrt", "exp", "sin", "cos"):
            a = self.emit(e.args[0], scope)
            code = {"sqr": SQR, "sqrt": SQRT, "exp": EXP, "sin": SIN, "cos": COS}[op]
            ctx.ins.append(_Ins(code, v, a, 0, 0, 0, (a,), v))
        elif op in ("sum", "prod"):
            if scope is not None:
                raise CodeListError("a Sum/Prod inside a Sum/Prod body must not be nested")
            body, lo, hi, init = e.args
            n = ctx.n
            hi = n if hi is None else (hi + n if hi < 0 else hi)
            lo = lo + n if lo < 0 else lo
            acc0 = self.emit(init, None)
            if not 0 <= lo <= hi <= n:
                raise CodeListError(f"loop range {lo}..{hi} outside 0..{n}")
            if lo == hi:
                self.done[key] = acc0
                return acc0
            offs: set = set()
            if ctx.use_tables and _table_offsets(body, offs) and len(offs) <= MAX_TABLE_OFFSETS and (
                    len(ctx.tables) < MAX_TABLES or (0 if op == "sum" else 1, lo, hi, body.key) in ctx.table_ix):
                t = ctx.table(0 if op == "sum" else 1, lo, hi, sorted(offs), body)
                ctx.ins.append(_Ins(TRED, v, acc0, 0, t, 0, (acc0,), v))
                self.done[key] = v
                return v
            # loop-invariant parts of the body first
            self._hoist(body, (lo, hi))
            ctx.ins.append(_Ins(MOV, v, acc0, 0, 0, 0, (acc0,), v))
            ctx.ins.append(_Ins(LOOP, 0, 0, 0, lo, hi))
            t = self.emit(body, (lo, hi))
            ctx.ins.append(_Ins(ADD if op == "sum" else MUL, v, v, t, 0, 0, (v, t), v))
            ctx.ins.append(_Ins(ENDLOOP))
            # values computed inside the loop are not visible after it
            for k in [k for k in self.done if k[1] == (lo, hi)]:
                del self.done[k]
        else:
            raise CodeListError(f"unknown operation {op}")
        self.done[key] = v
        return v

    def _hoist(self, e, scope):
        if not isinstance(e, Expr):
            return
        if not _depends(e, BASE_I, self.dep):
            self.emit(e, None)
            return
        for a in e.args:
            if isinstance(a, Expr):
                self._hoist(a, scope)

    def _check_range(self, base: int, off: int, scope, length: int | None = None):
        n = self.ctx.n
        size = n if length is None else length
        if base == BASE_ABS:
            if not 0 <= off < size:
                raise CodeListError(f"index {off} outside 0..{size - 1}")
        elif base == BASE_I:
            if scope is None:
                raise CodeListError("the loop index is used outside Sum/Prod")
            lo, hi = scope
            if lo + off < 0 or hi - 1 + off >= size:
                raise CodeListError(f"i{off:+d} leaves 0..{size - 1} for i in {lo}..{hi - 1}")
        elif base == BASE_J:
            if self.section < 0:
                raise CodeListError("the gradient coordinate j is used outside a gradient section")
            lo, hi = self.sec_range
            if lo + off < 0 or hi - 1 + off >= size:
                raise CodeListError(f"j{off:+d} leaves 0..{size - 1} for j in {lo}..{hi - 1}")


def _allocate(ins: list[_Ins], keep_until: dict[int, int]) -> int:
    """Linear-scan register allocation over the straight code.  A value defined
    before a loop and read inside it stays live to the loop's end."""
    last: dict[int, int] = {}
    loops = []
    start = None
    for p, t in enumerate(ins):
        if t.op == LOOP:
            start = p
        elif t.op == ENDLOOP:
            loops.append((start, p))
        for r in t.reads:
            last[r] = p
    defs: dict[int, int] = {}
    for p, t in enumerate(ins):
        if t.writes >= 0 and t.writes not in defs:
            defs[t.writes] = p
    for v, d in defs.items():
        lu = max(last.get(v, d), keep_until.get(v, -1))
        for ls, le in loops:
            if d < ls and ls < lu <= le:
                lu = le
            # an accumulator written inside the loop and read after it
        last[v] = lu
    # accumulators (written inside the loop, defined before it) also span the loop
    for ls, le in loops:
        for p in range(ls, le + 1):
            w = ins[p].writes
            if w >= 0 and defs[w] < ls:
                last[w] = max(last[w], le)
    reg: dict[int, int] = {}
    free = list(range(MAX_REGS))
    active: list[tuple[int, int]] = []  # (last use, value)
    nreg = 0
    for p, t in enumerate(ins):
        if t.writes < 0 or t.writes in reg:
            continue
        # release registers whose value is dead before this instruction writes
        keep = []
        for lu, v in active:
            if lu < p or (lu == p and v in t.reads):
                free.append(reg[v])
            else:
                keep.append((lu, v))
        active = keep
        if not free:
            raise CodeListError(f"the code list needs more than {MAX_REGS} interval registers")
        free.sort()
        r = free.pop(0)
        reg[t.writes] = r
        nreg = max(nreg, r + 1)
        active.append((last[t.writes], t.writes))
    for t in ins:
        if t.op in (LOOP, ENDLOOP):
            continue
        t.dst = reg[t.writes]
        if t.op in (ADD, MINUS, MUL, DIV):
            t.a, t.b = reg[t.a], reg[t.b]
        elif t.op in (TIMES, PLUS, TIMESK, PLUSK, SQR, SQRT, EXP, SIN, COS, MOV, TRED):
            t.a = reg[t.a]
    return nreg, reg


@dataclass
class CompiledCodeList:
    coef: np.ndarray
    n: int
    nreg: int
    instructions: int

    def disassemble(self) -> str:
        return disassemble(self.coef)


def compile_objective(f: Expr, n: int, gradient: Gradient | str | None = None,
                      tables: bool = True) -> CompiledCodeList:
    """Compile the value expression (and optionally the gradient code list) for
    dimension n into a ``GPUGO_CODELIST`` coefficient array.  ``gradient="auto"``
    derives the gradient symbolically (:func:`auto_gradient`); ``tables=False``
    runs every reduction as a loop (same results, for checks)."""
    if not isinstance(f, Expr):
        raise CodeListError("the objective must be an expression")
    if n < 1:
        raise CodeListError("n must be positive")
    if isinstance(gradient, str):
        if gradient != "auto":
            raise CodeListError("gradient must be a Gradient, \"auto\" or None")
        gradient = auto_gradient(f, n)
    ctx = _Ctx(n, use_tables=tables)
    em = _Emitter(ctx)
    res = em.emit(f, None)
    val_len = len(ctx.ins)
    keep: dict[int, int] = {res: val_len - 1}
    sections = []
    pro_start = val_len
    pro_len = 0
    skip = NO_SKIP
    if gradient is not None:
        if gradient.skip_if_contains is not None:
            skip = ctx.const(_bits(float(gradient.skip_if_contains)))
        gem = _Emitter(ctx)
        secs = []
        for s in gradient.sections:
            hi = n if s.hi is None else (s.hi + n if s.hi < 0 else s.hi)
            lo = s.lo + n if s.lo < 0 else s.lo
            if not 0 <= lo < hi <= n:
                raise CodeListError(f"gradient section {lo}..{hi} outside 0..{n}")
            if lo + s.check < 0 or hi - 1 + s.check >= n:
                raise CodeListError("the KKT check offset leaves the coordinates")
            e = s.expr(_J)
            if not isinstance(e, Expr):
                raise CodeListError("a gradient section must return an expression")
            sk = s.skip_infinite(_J) if s.skip_infinite is not None else None
            if sk is not None and not isinstance(sk, Expr):
                raise CodeListError("skip_infinite must return an expression")
            offs: set = {s.check}
            tabled = (tables and len(secs) < MAX_TABLED_SECTIONS and _section_offsets(e, offs)
                      and (sk is None or _section_offsets(sk, offs)) and len(offs) <= MAX_SECTION_OFFSETS)
            secs.append((lo, hi, s, e, sk, sorted(offs) if tabled else None))
        covered = np.zeros(n, dtype=int)
        for lo, hi, _, _, _, _ in secs:
            covered[lo:hi] += 1
        if np.any(covered > 1):
            raise CodeListError("gradient sections overlap")
        # prologue: every maximal sub-expression of the sections that does not
        # read j, evaluated once per box
        dep: dict = {}
        pro_vals: list[int] = []

        def hoist(e):
            if not isinstance(e, Expr):
                return
            if not _depends(e, BASE_J, dep):
                pro_vals.append(gem.emit(e, None))
                return
            if e.op in ("sum", "prod"):
                raise CodeListError("a Sum/Prod that reads j is not supported in a gradient")
            for a in e.args:
                if isinstance(a, Expr):
                    hoist(a)

        for _, _, _, e, sk, toffs in secs:
            if toffs is not None:
                continue           # tabled sections are self-contained
            hoist(e)
            if sk is not None:
                hoist(sk)
        pro_len = len(ctx.ins) - pro_start
        for si, (lo, hi, s, e, sk, toffs) in enumerate(secs):
            start = len(ctx.ins)
            em_s = gem if toffs is None else _Emitter(ctx)   # tabled: nothing from the prologue
            em_s.section = si
            em_s.sec_range = (lo, hi)
            saved = dict(em_s.done)      # section-local values are not shared
            r = em_s.emit(e, None)
            rs = em_s.emit(sk, None) if sk is not None else None
            em_s.done = saved
            sections.append([lo, hi, start, len(ctx.ins) - start, r, s.check, rs, toffs])
        # the sections run once per coordinate: prologue values stay live past
        # the last section instruction
        end = len(ctx.ins)
        for v in pro_vals:
            keep[v] = max(keep.get(v, -1), end)
        for sec in sections:
            last = max(sec[2] + sec[3] - 1, pro_start + pro_len - 1)
            for v in (sec[4], sec[6]):
                if v is not None:
                    keep[v] = max(keep.get(v, -1), last)
    # The value program and the gradient are allocated separately (the value
    # result is dead before the gradient starts).
    nreg_v, reg_v = _allocate(ctx.ins[:val_len], {k: v for k, v in keep.items() if v < val_len})
    nreg_g = 0
    if gradient is not None:
        nreg_g, reg_g = _allocate(ctx.ins[val_len:], {k: v - val_len for k, v in keep.items() if v >= val_len})
        for sec in sections:
            sec[4] = reg_g[sec[4]]
            sec[6] = NO_REG if sec[6] is None else reg_g[sec[6]]
    # term-table bodies follow the value and gradient code
    tabs = []
    all_ins = list(ctx.ins)
    for t in ctx.tables:
        tabs.append([t["lo"], t["hi"], t["kind"], len(t["offs"])] + (t["offs"] + [0, 0])[:2] +
                    [0, len(all_ins), len(t["ins"]), t["reg"]])
        all_ins += t["ins"]
    nreg = max([nreg_v, nreg_g, 1] + [t["nreg"] for t in ctx.tables])
    coef = _pack(n, nreg, all_ins, ctx.consts, reg_v[res], val_len, pro_start, pro_len, sections, skip, tabs)
    return CompiledCodeList(coef, n, nreg, len(all_ins))


def _pack(n, nreg, ins, consts, res_reg, val_len, pro_start, pro_len, sections, skip, tabs) -> np.ndarray:
    words = [MAGIC, n, nreg, len(ins), len(consts), 0, val_len, pro_start, pro_len, len(sections), skip, res_reg,
             len(tabs), 0, 0, 0]
    for lo, hi, start, ln, r, chk, rs, toffs in sections:
        offs = (toffs or []) + [0, 0, 0]
        words += [lo, hi, start, ln, r, chk & 0xFFFFFFFF, rs, 1 if toffs else 0, len(toffs or []),
                  offs[0] & 0xFFFFFFFF, offs[1] & 0xFFFFFFFF, offs[2] & 0xFFFFFFFF]
    for lo, hi, kind, noff, o0, o1, _, start, ln, r in tabs:
        words += [lo, hi, kind, noff, o0 & 0xFFFFFFFF, o1 & 0xFFFFFFFF, 0, start, ln, r, 0, 0]
    for t in ins:
        words += [t.op | (t.dst << 8) | (t.a << 16) | (t.b << 24), t.imm1 & 0xFFFFFFFF, t.imm2 & 0xFFFFFFFF, 0]
    w = np.array(words, dtype=np.uint64)
    c = np.array(consts, dtype=np.uint64)
    return np.concatenate([w, c]).view(np.float64).copy()


def _words(coef: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(coef, dtype=np.float64).view(np.uint64)


def parse(coef: np.ndarray) -> dict:
    """Header, sections, term tables, instructions and constants of a compiled array."""
    w = _words(coef)
    if w.size < HEADER or int(w[0]) != MAGIC:
        raise CodeListError("not a code list")
    n, nreg, nins, ncst, vs, vl, ps, pl, nsec, skip, res, ntab = (int(x) for x in w[1:13])
    s32 = lambda u: u - (1 << 32) if u >= 1 << 31 else u
    u0 = HEADER + SEC_WORDS * nsec
    i0 = u0 + TAB_WORDS * ntab
    c0 = i0 + INS_WORDS * nins
    if w.size < c0 + ncst:
        raise CodeListError("code list truncated")
    secs = []
    for k in range(nsec):
        lo, hi, st, ln, r, chk, sk, tb, no, o0, o1, o2 = (int(x) for x in w[HEADER + SEC_WORDS * k:
                                                                           HEADER + SEC_WORDS * (k + 1)])
        secs.append(dict(lo=lo, hi=hi, start=st, len=ln, reg=r, check=s32(chk), skip_reg=sk,
                         tabled=[s32(o0), s32(o1), s32(o2)][:no] if tb else None))
    tabs = []
    for k in range(ntab):
        q = [int(x) for x in w[u0 + TAB_WORDS * k:u0 + TAB_WORDS * (k + 1)]]
        tabs.append(dict(lo=q[0], hi=q[1], kind=q[2], offs=[s32(q[4]), s32(q[5])][:q[3]], start=q[7], len=q[8],
                         reg=q[9]))
    ins = []
    for t in range(nins):
        a0, a1, a2 = (int(x) for x in w[i0 + INS_WORDS * t:i0 + INS_WORDS * t + 3])
        ins.append((a0 & 255, (a0 >> 8) & 255, (a0 >> 16) & 255, (a0 >> 24) & 255, s32(a1), s32(a2)))
    consts = np.ascontiguousarray(coef, dtype=np.float64)[c0:c0 + ncst].copy()
    return dict(n=n, nreg=nreg, value=(vs, vl), result=res, prologue=(ps, pl), sections=secs, tables=tabs,
                skip=skip, instructions=ins, consts=consts)


def disassemble(coef: np.ndarray) -> str:
    p = parse(coef)
    out = [f"n={p['n']} registers={p['nreg']} constants={len(p['consts'])}"]
    base = {BASE_ABS: "", BASE_I: "i", BASE_J: "j"}

    def ix(b, o):
        return f"{base[b]}{o:+d}" if b else f"{o}"

    for t, (op, d, a, b, i1, i2) in enumerate(p["instructions"]):
        name = OP_NAMES.get(op, f"op{op}")
        if op == LDX:
            s = f"r{d} = X[{ix(a, i1)}]"
        elif op in (LDC, TIMES, PLUS):
            c = float(p["consts"][i2])
            s = f"r{d} = {c!r}" if op == LDC else f"r{d} = {name.lower()}(r{a}, {c!r})"
        elif op == LDI:
            s = f"r{d} = [{float(p['consts'][i2])!r}, {float(p['consts'][i2 + 1])!r}]"
        elif op in (LDK, LDKI):
            s = f"r{d} = {name.lower()}(c{i2}[{ix(a, i1)}])"
        elif op in (TIMESK, PLUSK):
            s = f"r{d} = {name.lower()[:-1]}(r{a}, c{i2}[{ix(b, i1)}])"
        elif op in (ADD, MINUS, MUL, DIV):
            s = f"r{d} = {name.lower()}(r{a}, r{b})"
        elif op == LOOP:
            s = f"for i in {i1}..{i2 - 1}:"
        elif op == ENDLOOP:
            s = "end"
        elif op == TRED:
            tb = p["tables"][i1]
            s = f"r{d} = {'sum' if tb['kind'] == 0 else 'prod'}(r{a}, table {i1})"
        else:
            s = f"r{d} = {name.lower()}(r{a})"
        out.append(f"{t:4d}  {s}")
    vs, vl = p["value"]
    ps, pl = p["prologue"]
    out.append(f"value {vs}..{vs + vl - 1} (result r{p['result']}); gradient prologue {ps}..{ps + pl - 1}")
    for s in p["sections"]:
        sk = "" if s["skip_reg"] == NO_REG else f", no test when r{s['skip_reg']} has an infinite end"
        tb = "" if s["tabled"] is None else f", tabled over X[j{s['tabled']}]"
        out.append(f"section j in {s['lo']}..{s['hi'] - 1}: code {s['start']}..{s['start'] + s['len'] - 1}, "
                   f"gradient r{s['reg']}, KKT bounds of j{s['check']:+d}{sk}{tb}")
    if p["skip"] != NO_SKIP:
        out.append(f"skip the gradient test when every coordinate contains {float(p['consts'][p['skip']])!r}")
    for k, t in enumerate(p["tables"]):
        out.append(f"table {k}: {'sum' if t['kind'] == 0 else 'product'} over i in {t['lo']}..{t['hi'] - 1} of "
                   f"code {t['start']}..{t['start'] + t['len'] - 1} (r{t['reg']}), reads X[i{t['offs']}]")
    return "\n".join(out)


def point_value(coef: np.ndarray, x: Sequence[float]) -> float:
    """Plain FP64 evaluation (round to nearest, no interval arithmetic) of the
    value code list at a point, for checks."""
    p = parse(coef)
    n = p["n"]
    x = np.asarray(x, dtype=np.float64)
    if x.size != n:
        raise CodeListError("point of the wrong dimension")
    c = p["consts"]
    ins = p["instructions"]

    def run(start, length, R, i0=0):
        pc, i, hi, body = start, i0, 0, 0

        def idx(b, o):
            return (0 if b == BASE_ABS else i) + o

        while pc < start + length:
            op, d, a, b, i1, i2 = ins[pc]
            if op == LDX:
                R[d] = float(x[idx(a, i1)])
            elif op == LDC:
                R[d] = float(c[i2])
            elif op == LDI:
                R[d] = 0.5 * (float(c[i2]) + float(c[i2 + 1]))
            elif op == LDK:
                R[d] = float(c[i2 + idx(a, i1)])
            elif op == LDKI:
                k = i2 + 2 * idx(a, i1)
                R[d] = 0.5 * (float(c[k]) + float(c[k + 1]))
            elif op == ADD:
                R[d] = R[a] + R[b]
            elif op == MINUS:
                R[d] = R[a] - R[b]
            elif op == MUL:
                R[d] = R[a] * R[b]
            elif op == DIV:
                R[d] = R[a] / R[b] if R[b] != 0 else math.copysign(math.inf, R[a])
            elif op == TIMES:
                R[d] = R[a] * float(c[i2])
            elif op == PLUS:
                R[d] = R[a] + float(c[i2])
            elif op == TIMESK:
                R[d] = R[a] * float(c[i2 + idx(b, i1)])
            elif op == PLUSK:
                R[d] = R[a] + float(c[i2 + idx(b, i1)])
            elif op == SQR:
                R[d] = R[a] * R[a]
            elif op == SQRT:
                R[d] = math.sqrt(max(R[a], 0.0))
            elif op == EXP:
                R[d] = math.exp(R[a]) if R[a] < 709 else math.inf
            elif op == SIN:
                R[d] = math.sin(R[a])
            elif op == COS:
                R[d] = math.cos(R[a])
            elif op == MOV:
                R[d] = R[a]
            elif op == LOOP:
                i, hi, body = i1, i2, pc + 1
            elif op == ENDLOOP:
                i += 1
                if i < hi:
                    pc = body
                    continue
            elif op == TRED:
                t = p["tables"][i1]
                acc = R[a]
                for k in range(t["lo"], t["hi"]):
                    R2 = [0.0] * max(p["nreg"], 1)
                    run(t["start"], t["len"], R2, k)
                    acc = acc + R2[t["reg"]] if t["kind"] == 0 else acc * R2[t["reg"]]
                R[d] = acc
            pc += 1

    R = [0.0] * max(p["nreg"], 1)
    vs, vl = p["value"]
    run(vs, vl, R)
    return R[p["result"]]
