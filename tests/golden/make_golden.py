"""Generate the golden vectors in tests/golden/ from the GPUGO reference source.

Run in a container that has the reference checked out (it is read, never
modified or copied):

    python tests/golden/make_golden.py /path/to/GPUGO

The reference is Numba-CUDA code, and Numba is not installed here.  This script
executes the reference's own device functions as plain Python by providing a
stand-in ``numba`` module:

* ``cuda.jit`` returns the function unchanged;
* ``cuda.libdevice.dadd_rd/ru, dmul_rd/ru, ddiv_rd/ru, drcp_rd/ru`` round the
  exact rational result (``fractions.Fraction``) in the requested direction;
* ``cuda.libdevice.pow(x, 2)`` is ``x*x`` and ``pow(x, 0.5)`` is ``sqrt(x)``,
  both correctly rounded;
* ``cuda.libdevice.sin/cos/exp`` (closed libdevice code that is not in the
  reference) are the oracle's own functions, the same ones the CUDA product
  implements, so value and sample bounds are comparable bit for bit.

The scripts import their folder's old interval module (``import IARastrigin as
ia``); the stand-in maps that import to the reference's updated library
``Updated Interval Arithmetic Operations/IA.py``, whose directed-rounding
semantics the product follows.  Its ``times`` assumes a non-negative scalar
(IA.py:312) while the Ackley code list passes -0.02 and -20, so the Ackley and
Griewank vectors are generated with a sign-aware ``times``.

Only the imports and function definitions of each script are executed; its
top-level statements (the whole 50-variable B&B run) are skipped.  The result-box
merging vectors come from the same execution of ``rosenbrock50.py``'s host
functions ``combine`` / ``connectivity``.

``--levy10000`` adds the reference's largest script (10 000 variables) to it;
``--large`` writes ``reference_vectors_1000.npz`` from the four families'
1000-variable scripts, and ``--codelist-large`` writes
``codelist_vectors_1000.npz`` from the seven code-list benchmarks'
1000-variable scripts.

``--codelist`` writes ``codelist_vectors.npz`` instead: the value, sample and
derivative code lists of the seven scripts without a built-in family (Levy,
Salomon, Styblinski, Belegundu, Breiman, Fu, Zabinsky), which pin the code-list
interpreter.  Their scalar multiplications use the sign-aware ``times`` (two of
them pass -0.1 and -1).
"""
from __future__ import annotations

import ast
import math
import os
import sys
import time
import types
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
import oracle  # noqa: E402  (the oracle's transcendentals stand in for libdevice)

DBL_MAX = Fraction(sys.float_info.max)


def _round(q: Fraction, up: bool) -> float:
    if abs(q) > DBL_MAX:
        if q > 0:
            return math.inf if up else sys.float_info.max
        return -sys.float_info.max if up else -math.inf
    f = float(q)
    if Fraction(f) == q:
        return f
    if up:
        return f if Fraction(f) > q else float(np.nextafter(f, np.inf))
    return f if Fraction(f) < q else float(np.nextafter(f, -np.inf))


def _nonfinite(*xs):
    return any(not math.isfinite(float(x)) for x in xs)


def _dadd(a, b, up):
    a = float(a); b = float(b)
    if _nonfinite(a, b):
        return np.float64(a + b)
    q = Fraction(a) + Fraction(b)
    if q == 0:
        if a == 0 and b == 0:
            na, nb = math.copysign(1, a) < 0, math.copysign(1, b) < 0
            neg = (na and nb) if up else (na or nb)
            return np.float64(-0.0 if neg else 0.0)
        return np.float64(0.0 if up else -0.0)
    return np.float64(_round(q, up))


def _dmul(a, b, up):
    a = float(a); b = float(b)
    if _nonfinite(a, b) or a == 0 or b == 0:
        return np.float64(a * b)
    return np.float64(_round(Fraction(a) * Fraction(b), up))


def _ddiv(a, b, up):
    a = float(a); b = float(b)
    if _nonfinite(a, b) or a == 0 or b == 0:
        with np.errstate(all="ignore"):
            return np.float64(np.float64(a) / np.float64(b))
    return np.float64(_round(Fraction(a) / Fraction(b), up))


def _pow(x, p):
    x = np.float64(x)
    if p == 2:
        return np.float64(x * x)
    if p == 0.5:
        return np.float64(np.sqrt(x))
    raise ValueError(f"pow exponent {p} not used by the four families")


def _point(fn):
    def f(x):
        return np.float64(oracle.point_fn(fn, np.array([float(x)]))[0])
    return f


def make_numba_stub():
    numba = types.ModuleType("numba")
    cuda = types.SimpleNamespace()

    def jit(*args, **kwargs):
        if args and callable(args[0]):
            return args[0]
        return lambda f: f

    lib = types.SimpleNamespace(
        dadd_rd=lambda a, b: _dadd(a, b, False), dadd_ru=lambda a, b: _dadd(a, b, True),
        dmul_rd=lambda a, b: _dmul(a, b, False), dmul_ru=lambda a, b: _dmul(a, b, True),
        ddiv_rd=lambda a, b: _ddiv(a, b, False), ddiv_ru=lambda a, b: _ddiv(a, b, True),
        drcp_rd=lambda b: _ddiv(1.0, b, False), drcp_ru=lambda b: _ddiv(1.0, b, True),
        pow=_pow, sin=_point("sin"), cos=_point("cos"), exp=_point("exp"))
    cuda.jit = jit
    cuda.libdevice = lib
    numba.cuda = cuda
    return numba


def load_updated_ia(ref_root: str, sign_aware_times: bool):
    path = os.path.join(ref_root, "Updated Interval Arithmetic Operations", "IA.py")
    mod = types.ModuleType("IA_updated")
    mod.__file__ = path
    exec(compile(open(path).read(), path, "exec"), mod.__dict__)
    if sign_aware_times:
        dmul_rd, dmul_ru = mod.cuda.libdevice.dmul_rd, mod.cuda.libdevice.dmul_ru

        def times(lower, upper, val):
            if val < 0:
                return dmul_rd(upper, val), dmul_ru(lower, val)
            return dmul_rd(lower, val), dmul_ru(upper, val)
        mod.times = times
    return mod


def load_script(ref_root: str, rel: str, ia_name: str, ia_mod):
    """Execute the function definitions of one reference script."""
    path = os.path.join(ref_root, rel)
    src = open(path).read()
    tree = ast.parse(src)
    keep = [node for node in tree.body
            if isinstance(node, (ast.Import, ast.ImportFrom, ast.FunctionDef))]
    sys.modules[ia_name] = ia_mod
    ns: dict = {"__name__": "ref_" + ia_name}
    exec(compile(ast.Module(body=keep, type_ignores=[]), path, "exec"), ns)
    return ns


FAMILIES = {
    # name: (script, ia module name, prefix, domain, family id, coef builder, sign-aware times)
    "rastrigin": ("GPUGO_1.1/7-Rastrigin/rastrigin50.py", "IARastrigin", "rastrigin", (-5.5, 6.0), 1,
                  lambda n: np.concatenate([np.ones(n), np.full(n, 10.0), np.ones(n)]), False),
    "rosenbrock": ("GPUGO_1.1/11-Rosenbrock/rosenbrock50.py", "IARosenbrock", "rosenbrock", (-30.0, 30.0), 2,
                   lambda n: np.concatenate([np.full(n - 1, 100.0), np.ones(n - 1)]), False),
    "ackley": ("GPUGO_1.1/1-Ackley/ackley50.py", "IAAckley", "ackley", (-35.0, 40.0), 3,
               lambda n: np.concatenate([[20.0, 0.02], np.ones(n)]), True),
    "griewank": ("GPUGO_1.1/5-Griewank/griewank50.py", "IAGriewank", "griewank", (-100.0, 110.0), 4,
                 lambda n: np.array([4000.0]), True),
}
N = 50
WID, GROUP, SAMPLES = 4, 10, 10


def parents_for(name, dom, complete, rng):
    """Parent boxes: the domain, one of its children, and a small box around the minimiser."""
    lo, hi = dom
    root = np.tile([lo, hi], N).astype(np.float64)
    c1 = complete(root, int(rng.integers(0, WID ** GROUP)), 1)
    xstar = 1.0 if name == "rosenbrock" else 0.0
    tiny = np.empty(2 * N)
    for i in range(N):
        w = float(rng.uniform(0.5, 2.0)) * 1e-3
        off = float(rng.uniform(-0.4, 0.4)) * w
        tiny[2 * i] = xstar - w + off
        tiny[2 * i + 1] = xstar + w + off
    return [(root, 1), (c1, 11), (tiny, 41)]


def main(ref_root: str):
    oracle.build()
    sys.modules["numba"] = make_numba_stub()
    rng = np.random.default_rng(0x6770756F)
    out = {}
    for name, (rel, ia_name, pre, dom, fam, coef, sign_times) in FAMILIES.items():
        ia_mod = load_updated_ia(ref_root, sign_times)
        ns = load_script(ref_root, rel, ia_name, ia_mod)
        value = ns[pre + "Value_IA"]
        sample = ns[pre + "Sample_IA"]
        deriv = ns[pre + "Derivative_IA"]
        complete = ns["completeRegion"]
        select = ns["selectVarInSubRegion"]
        parents = parents_for(name, dom, complete, rng)
        pidx, cycs, codes, lbs, flags, samps, dflags = [], [], [], [], [], [], []
        for k, (pbox, cyc) in enumerate(parents):
            pos = [int(p) for p in rng.integers(0, WID ** GROUP, 40)] + [0, WID ** GROUP - 1]
            for p in pos:
                lb, _ = value(pbox, p, 1e300, 0, cyc)
                lb = float(lb)
                # ruleOut value test against a UB just below the LB: must flag 1
                _, f_lo = value(pbox, p, lb - abs(lb) * 1e-9 - 1e-300, 0, cyc)
                lbs.append(lb)
                flags.append(int(f_lo))
                samps.append(float(sample(pbox, p, SAMPLES, cyc)))
                # the Ackley gradient code list is not reproduced (see the oracle header)
                dflags.append(int(deriv(pbox, p, 0, cyc)) if name != "ackley" else -1)
                pidx.append(k); cycs.append(cyc); codes.append(p)
        out[name + "_family"] = np.array([fam])
        out[name + "_coef"] = coef(N)
        out[name + "_domain"] = np.tile(np.array(dom, dtype=np.float64), N)
        out[name + "_parents"] = np.stack([pb for pb, _ in parents])
        out[name + "_parent_idx"] = np.array(pidx, dtype=np.int64)
        out[name + "_cyc"] = np.array(cycs, dtype=np.int64)
        out[name + "_code"] = np.array(codes, dtype=np.int64)
        out[name + "_lb"] = np.array(lbs)
        out[name + "_flag_below"] = np.array(flags, dtype=np.int64)
        out[name + "_samp"] = np.array(samps)
        out[name + "_dflag"] = np.array(dflags, dtype=np.int64)
        print(name, "cases", len(codes), flush=True)
        if name == "rastrigin":
            # box decoder: completeRegion and selectVarInSubRegion on the parents above
            dec_par, dec_cyc, dec_code, dec_box, dec_sel = [], [], [], [], []
            for t in range(60):
                pbox = parents[t % 3][0]
                cyc = int(rng.choice([1, 11, 21, 31, 41]))
                p = int(rng.integers(0, WID ** GROUP))
                box = complete(pbox, p, cyc)
                sel = np.array([select(pbox, i, p, cyc) for i in range(1, N + 1)], dtype=np.float64).ravel()
                dec_par.append(t % 3); dec_cyc.append(cyc); dec_code.append(p)
                dec_box.append(np.asarray(box, dtype=np.float64)); dec_sel.append(sel)
            out["decoder_parent_idx"] = np.array(dec_par)
            out["decoder_cyc"] = np.array(dec_cyc)
            out["decoder_code"] = np.array(dec_code)
            out["decoder_complete"] = np.stack(dec_box)
            out["decoder_select"] = np.stack(dec_sel)
    out.update(combine_cases(ref_root))
    dst = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)


def combine_cases(ref_root: str) -> dict:
    """Result-box merging: the reference's host functions ``combine`` and
    ``connectivity`` (rosenbrock50.py:926-1049) run on sequences of small boxes,
    some within the combine tolerance of each other, some not."""
    ia_mod = load_updated_ia(ref_root, False)
    ns = load_script(ref_root, FAMILIES["rosenbrock"][0], "IARosenbrock", ia_mod)
    combine = ns["combine"]
    rng = np.random.default_rng(0x636F6D62)
    ns_, tols, boxes, boff, roots, roff = [], [], [], [0], [], [0]
    for case in range(24):
        n = int(rng.choice([1, 2, 3, 5, 8]))
        tol = float(rng.choice([1e-3, 1e-4]))
        centres = rng.uniform(-2.0, 2.0, size=(int(rng.integers(1, 4)), n))
        seq = []
        for _ in range(int(rng.integers(1, 40))):
            c = centres[int(rng.integers(0, len(centres)))]
            lo = c + rng.uniform(-3.0, 3.0, size=n) * tol
            w = rng.choice([0.01, 0.1, 0.5, 2.0]) * tol * rng.uniform(0.5, 1.0, size=n)
            box = np.empty(2 * n)
            box[0::2] = lo
            box[1::2] = lo + w
            if seq and rng.random() < 0.15:          # a box inside an earlier one
                prev = seq[int(rng.integers(0, len(seq)))]
                box = prev.copy()
                box[0::2] += 0.25 * (prev[1::2] - prev[0::2])
                box[1::2] -= 0.25 * (prev[1::2] - prev[0::2])
            seq.append(box)
        combined: list = []
        for box in seq:
            combine(box.copy(), combined, tol)
        ns_.append(n); tols.append(tol)
        boxes.extend(seq); boff.append(boff[-1] + len(seq))
        roots.extend(np.asarray(r, dtype=np.float64) for r in combined); roff.append(roff[-1] + len(combined))
    flat = lambda arrs: np.concatenate([np.asarray(a, dtype=np.float64).ravel() for a in arrs])
    print("combine cases", len(ns_), "boxes", len(boxes), "roots", len(roots), flush=True)
    return {"combine_n": np.array(ns_, dtype=np.int64), "combine_tol": np.array(tols),
            "combine_box_offsets": np.array(boff, dtype=np.int64), "combine_boxes": flat(boxes),
            "combine_root_offsets": np.array(roff, dtype=np.int64), "combine_roots": flat(roots)}


CODELIST_SCRIPTS = {
    # name: (script, ia module name, function prefix, domain, centre of the small parent box)
    # (its width is 1 % of the domain, or SMALL_WIDTH[name])
    "levy": ("GPUGO_1.1/6-Levy/levy50.py", "IALevy", "Levy", (-10.0, 10.0), -3.0),
    "salomon": ("GPUGO_1.1/8-Salomon/salomon50.py", "IASalomon", "salomon", (-100.0, 110.0), 30.0),
    "corrupted": ("GPUGO_1.1/9-Styblinski/corrupted50.py", "IACorrupted", "corrupted", (-10.0, 11.0), 0.0),
    "deflected": ("GPUGO_1.1/2-Belegundu/deflected50.py", "IADeflected", "deflected", (-10.0, 11.0), 5.0),
    "cosine": ("GPUGO_1.1/3-Breiman/cosine50.py", "IACosine", "cosine", (-1.0, 2.0), 0.0),
    "trigonometric": ("GPUGO_1.1/4-Fu/trigonometric50.py", "IATrigonometric", "trigonometric", (-10.0, 10.0), 0.9),
    "sinusoidal": ("GPUGO_1.1/10-Zabinsky/sinusoidal50.py", "IASinusoidal", "sinusoidal", (0.0, math.pi),
                   2.0 * math.pi / 3),
}
CODELIST_PER_PARENT = 40
SMALL_WIDTH = {"salomon": 1e-8}   # the Salomon gradient excludes 0 only on very small boxes


def codelist_main(ref_root: str, only: list[str] | None = None):
    oracle.build()
    sys.modules["numba"] = make_numba_stub()
    rng = np.random.default_rng(0x636C6973)
    dst = os.path.join(HERE, "codelist_vectors.npz")
    out = dict(np.load(dst)) if (only and os.path.exists(dst)) else {}
    for name, (rel, ia_name, pre, dom, centre) in CODELIST_SCRIPTS.items():
        sub = np.random.default_rng(rng.integers(1 << 62))   # per script, so one can be regenerated alone
        if only and name not in only:
            continue
        ia_mod = load_updated_ia(ref_root, True)
        ns = load_script(ref_root, rel, ia_name, ia_mod)
        value, sample, deriv = ns[pre + "Value_IA"], ns[pre + "Sample_IA"], ns[pre + "Derivative_IA"]
        complete = ns["completeRegion"]
        lo, hi = dom
        root = np.tile([lo, hi], N).astype(np.float64)
        c1 = complete(root, int(sub.integers(0, WID ** GROUP)), 1)
        c1 = np.asarray(c1, dtype=np.float64)
        small = np.empty(2 * N)
        for i in range(N):
            w = float(sub.uniform(0.5, 2.0)) * SMALL_WIDTH.get(name, 1e-2) * (hi - lo)
            off = float(sub.uniform(-0.4, 0.4)) * w
            small[2 * i] = max(lo, centre - w + off)
            small[2 * i + 1] = min(hi, centre + w + off)
        parents = [(root, 1), (c1, 11), (small, 41)]
        pidx, cycs, codes, lbs, samps, dflags = [], [], [], [], [], []
        t0 = time.time()
        for k, (pbox, cyc) in enumerate(parents):
            pos = [int(v) for v in sub.integers(0, WID ** GROUP, CODELIST_PER_PARENT - 2)] + [0, WID ** GROUP - 1]
            for q in pos:
                lb, _ = value(pbox, q, 1e300, 0, cyc)
                lbs.append(float(lb))
                samps.append(float(sample(pbox, q, SAMPLES, cyc)))
                dflags.append(int(deriv(pbox, q, 0, cyc)))
                pidx.append(k); cycs.append(cyc); codes.append(q)
        out[name + "_domain"] = np.tile(np.array(dom, dtype=np.float64), N)
        out[name + "_parents"] = np.stack([pb for pb, _ in parents])
        out[name + "_parent_idx"] = np.array(pidx, dtype=np.int64)
        out[name + "_cyc"] = np.array(cycs, dtype=np.int64)
        out[name + "_code"] = np.array(codes, dtype=np.int64)
        out[name + "_lb"] = np.array(lbs)
        out[name + "_samp"] = np.array(samps)
        out[name + "_dflag"] = np.array(dflags, dtype=np.int64)
        print(name, "cases", len(codes), f"{time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(dst, **out)
    print("wrote", dst)


def large_main(ref_root: str, n: int = 1000):
    """The four families' 1000-variable scripts (rastrigin1000.py, ...): the same
    device functions at the reference's larger size, written to
    reference_vectors_1000.npz (12 children per family at the first, a middle
    and the last cycle)."""
    oracle.build()
    sys.modules["numba"] = make_numba_stub()
    rng = np.random.default_rng(0x6C617267)
    out = {}
    for name, (rel, ia_name, pre, dom, fam, coef, sign_times) in FAMILIES.items():
        rel_n = rel.replace("50.py", f"{n}.py")
        ia_mod = load_updated_ia(ref_root, sign_times)
        ns = load_script(ref_root, rel_n, ia_name, ia_mod)
        value, sample, deriv = ns[pre + "Value_IA"], ns[pre + "Sample_IA"], ns[pre + "Derivative_IA"]
        complete = ns["completeRegion"]
        lo, hi = dom
        root = np.tile([lo, hi], n).astype(np.float64)
        mid_cyc = 1 + GROUP * (n // (2 * GROUP))
        last_cyc = n - GROUP + 1
        c1 = np.asarray(complete(root, int(rng.integers(0, WID ** GROUP)), 1), dtype=np.float64)
        xstar = 1.0 if name == "rosenbrock" else 0.0
        small = np.empty(2 * n)
        for i in range(n):
            w = float(rng.uniform(0.5, 2.0)) * 1e-3
            off = float(rng.uniform(-0.4, 0.4)) * w
            small[2 * i], small[2 * i + 1] = xstar - w + off, xstar + w + off
        parents = [(root, 1), (c1, mid_cyc), (small, last_cyc)]
        pidx, cycs, codes, lbs, samps, dflags = [], [], [], [], [], []
        t0 = time.time()
        for k, (pbox, cyc) in enumerate(parents):
            for q in [int(v) for v in rng.integers(0, WID ** GROUP, 3)] + [WID ** GROUP - 1]:
                lb, _ = value(pbox, q, 1e300, 0, cyc)
                lbs.append(float(lb))
                samps.append(float(sample(pbox, q, SAMPLES, cyc)))
                dflags.append(int(deriv(pbox, q, 0, cyc)) if name != "ackley" else -1)
                pidx.append(k); cycs.append(cyc); codes.append(q)
        out[name + "_family"] = np.array([fam])
        out[name + "_coef"] = coef(n)
        out[name + "_domain"] = np.tile(np.array(dom, dtype=np.float64), n)
        out[name + "_parents"] = np.stack([pb for pb, _ in parents])
        out[name + "_parent_idx"] = np.array(pidx, dtype=np.int64)
        out[name + "_cyc"] = np.array(cycs, dtype=np.int64)
        out[name + "_code"] = np.array(codes, dtype=np.int64)
        out[name + "_lb"] = np.array(lbs)
        out[name + "_samp"] = np.array(samps)
        out[name + "_dflag"] = np.array(dflags, dtype=np.int64)
        print(name, n, "cases", len(codes), f"{time.time() - t0:.0f} s", flush=True)
    dst = os.path.join(HERE, f"reference_vectors_{n}.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)


def codelist_large_main(ref_root: str, n: int = 1000):
    """The seven code-list benchmarks' 1000-variable scripts (levy1000.py,
    salomon1000.py, ...): value, sample and derivative of 12 children per script
    at the first, a middle and the last cycle, written to
    codelist_vectors_1000.npz."""
    oracle.build()
    sys.modules["numba"] = make_numba_stub()
    rng = np.random.default_rng(0x636C3130)
    out = {}
    for name, (rel, ia_name, pre, dom, centre) in CODELIST_SCRIPTS.items():
        ia_mod = load_updated_ia(ref_root, True)
        ns = load_script(ref_root, rel.replace("50.py", f"{n}.py"), ia_name, ia_mod)
        value, sample, deriv = ns[pre + "Value_IA"], ns[pre + "Sample_IA"], ns[pre + "Derivative_IA"]
        complete = ns["completeRegion"]
        lo, hi = dom
        root = np.tile([lo, hi], n).astype(np.float64)
        c1 = np.asarray(complete(root, int(rng.integers(0, WID ** GROUP)), 1), dtype=np.float64)
        small = np.empty(2 * n)
        for i in range(n):
            w = float(rng.uniform(0.5, 2.0)) * SMALL_WIDTH.get(name, 1e-2) * (hi - lo)
            off = float(rng.uniform(-0.4, 0.4)) * w
            small[2 * i] = max(lo, centre - w + off)
            small[2 * i + 1] = min(hi, centre + w + off)
        parents = [(root, 1), (c1, 1 + GROUP * (n // (2 * GROUP))), (small, n - GROUP + 1)]
        pidx, cycs, codes, lbs, samps, dflags = [], [], [], [], [], []
        t0 = time.time()
        for k, (pbox, cyc) in enumerate(parents):
            for q in [int(v) for v in rng.integers(0, WID ** GROUP, 3)] + [WID ** GROUP - 1]:
                lb, _ = value(pbox, q, 1e300, 0, cyc)
                lbs.append(float(lb))
                samps.append(float(sample(pbox, q, SAMPLES, cyc)))
                dflags.append(int(deriv(pbox, q, 0, cyc)))
                pidx.append(k); cycs.append(cyc); codes.append(q)
        out[name + "_domain"] = np.tile(np.array(dom, dtype=np.float64), n)
        out[name + "_parents"] = np.stack([pb for pb, _ in parents])
        out[name + "_parent_idx"] = np.array(pidx, dtype=np.int64)
        out[name + "_cyc"] = np.array(cycs, dtype=np.int64)
        out[name + "_code"] = np.array(codes, dtype=np.int64)
        out[name + "_lb"] = np.array(lbs)
        out[name + "_samp"] = np.array(samps)
        out[name + "_dflag"] = np.array(dflags, dtype=np.int64)
        print(name, n, "cases", len(codes), f"{time.time() - t0:.0f} s", flush=True)
    dst = os.path.join(HERE, f"codelist_vectors_{n}.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)


def levy10000_main(ref_root: str):
    """The reference's largest script, levy10000.py (10 000 variables, wid 4,
    cycles of 10): value, sample and derivative of a few children at the first
    cycle, a middle cycle and the last one, added to codelist_vectors.npz as
    levy10000_*.  Exact rational rounding over 10^5 operations per child makes
    this slow (minutes)."""
    oracle.build()
    sys.modules["numba"] = make_numba_stub()
    rng = np.random.default_rng(0x6C763130)
    n = 10000
    dst = os.path.join(HERE, "codelist_vectors.npz")
    out = dict(np.load(dst))
    ia_mod = load_updated_ia(ref_root, True)
    ns = load_script(ref_root, "GPUGO_1.1/6-Levy/levy10000.py", "IALevy", ia_mod)
    value, sample, deriv = ns["LevyValue_IA"], ns["LevySample_IA"], ns["LevyDerivative_IA"]
    complete = ns["completeRegion"]
    root = np.tile([-10.0, 10.0], n).astype(np.float64)
    mid = np.asarray(complete(root, int(rng.integers(0, WID ** GROUP)), 1), dtype=np.float64)
    parents = [(root, 1), (mid, 4001), (root, n - 9)]
    pidx, cycs, codes, lbs, samps, dflags = [], [], [], [], [], []
    t0 = time.time()
    for k, (pbox, cyc) in enumerate(parents):
        for q in [int(v) for v in rng.integers(0, WID ** GROUP, 3)] + [WID ** GROUP - 1]:
            lb, _ = value(pbox, q, 1e300, 0, cyc)
            lbs.append(float(lb))
            samps.append(float(sample(pbox, q, SAMPLES, cyc)))
            dflags.append(int(deriv(pbox, q, 0, cyc)))
            pidx.append(k); cycs.append(cyc); codes.append(q)
            print("levy10000 child", len(codes), f"{time.time() - t0:.0f} s", flush=True)
    out["levy10000_domain"] = np.tile(np.array([-10.0, 10.0]), n)
    out["levy10000_parents"] = np.stack([pb for pb, _ in parents])
    out["levy10000_parent_idx"] = np.array(pidx, dtype=np.int64)
    out["levy10000_cyc"] = np.array(cycs, dtype=np.int64)
    out["levy10000_code"] = np.array(codes, dtype=np.int64)
    out["levy10000_lb"] = np.array(lbs)
    out["levy10000_samp"] = np.array(samps)
    out["levy10000_dflag"] = np.array(dflags, dtype=np.int64)
    np.savez_compressed(dst, **out)
    print("wrote", dst)


# ---------------------------------------------------------------------------
# the reference's host loop, run as written on a reduced problem
# ---------------------------------------------------------------------------
# Text substitutions that shrink rastrigin50.py to 10 variables split in two
# parts each (2^10 = 1024 children per iteration, one cycle of 10 coordinates)
# and size its kernel grids to those 1024 children.  Each is applied exactly as
# many times as listed, or the run stops: the script's own logic is otherwise
# executed unchanged.
LOOP_SCRIPT = "GPUGO_1.1/7-Rastrigin/rastrigin50.py"
LOOP_N, LOOP_WID = 10, 2
LOOP_SUBS = [
    ("    n = 50 # The number of variables in the Rastrigin function", f"    n = {LOOP_N}", 3),
    ("    length = 50 # The number of variables in the Rastrigin function", f"    length = {LOOP_N}", 2),
    ("    wid = 4", f"    wid = {LOOP_WID}", 2),
    ("initialRegion = np.tile([-5.5, 6], 50)", f"initialRegion = np.tile([-5.5, 6], {LOOP_N})", 1),
    ("maximumCyc = 41", "maximumCyc = 1", 1),
    ("    blockspergridSample = 2048", "    blockspergridSample = 4", 1),
    ("    threadsperblockSample = 512", "    threadsperblockSample = 256", 1),
    ("    blockspergridRule = 4096", "    blockspergridRule = 4", 1),
]


class _LoopDone(Exception):
    pass


def make_kernel_runtime():
    """Stand-in for the parts of numba.cuda the host loop and its kernels use.
    A kernel launch runs every thread of the grid: one after another in thread
    order (the order the reference's atomic counters would take if its threads
    ran in order), or, for a kernel that synchronises its block, as one Python
    thread per CUDA thread with a barrier for cuda.syncthreads."""
    import threading
    tls = threading.local()

    class _Idx:
        def __init__(self, attr):
            self.attr = attr

        @property
        def x(self):
            return getattr(tls, self.attr)

    class DeviceArray(np.ndarray):
        def copy_to_host(self):
            return np.array(self)

    def to_device(a):
        return np.array(a).view(DeviceArray)

    def device_array(shape, dtype=np.float64):
        return np.zeros(shape, dtype=dtype).view(DeviceArray)

    class Kernel:
        def __init__(self, fn):
            self.fn = fn
            self.syncs = "syncthreads" in fn.__code__.co_names

        def __call__(self, *args):          # called from device code: a device function
            return self.fn(*args)

        def __getitem__(self, cfg):
            blocks, threads = cfg

            def launch(*args):
                for b in range(blocks):
                    shared = {}
                    if not self.syncs:
                        for t in range(threads):
                            tls.block, tls.thread, tls.dim, tls.shared, tls.barrier = b, t, threads, shared, None
                            self.fn(*args)
                        continue
                    barrier = threading.Barrier(threads)
                    errs = []

                    def body(t):
                        tls.block, tls.thread, tls.dim, tls.shared, tls.barrier = b, t, threads, shared, barrier
                        try:
                            self.fn(*args)
                        except Exception as e:      # surfaced after the block
                            errs.append(e)
                            barrier.abort()
                    ts = [threading.Thread(target=body, args=(t,)) for t in range(threads)]
                    for th in ts:
                        th.start()
                    for th in ts:
                        th.join()
                    if errs:
                        raise errs[0]
            return launch

    def jit(*args, **kwargs):
        if args and callable(args[0]):
            return Kernel(args[0])
        return lambda f: f                  # device functions run as plain Python

    _shared_lock = threading.Lock()

    def shared_array(shape, dtype):
        with _shared_lock:                  # one array per block, shared by its threads
            return tls.shared.setdefault(("a", shape), np.zeros(shape, dtype=dtype))

    def atomic_min(arr, i, v):
        old = arr[i]
        if v < old:
            arr[i] = v
        return old

    def atomic_add(arr, i, v):
        old = arr[i]
        arr[i] = old + v
        return old

    numba = make_numba_stub()
    cuda = numba.cuda
    cuda.jit = jit
    cuda.grid = lambda d: tls.block * tls.dim + tls.thread
    cuda.threadIdx = _Idx("thread")
    cuda.blockIdx = _Idx("block")
    cuda.blockDim = _Idx("dim")
    cuda.syncthreads = lambda: tls.barrier.wait()
    cuda.shared = types.SimpleNamespace(array=shared_array)
    cuda.atomic = types.SimpleNamespace(min=atomic_min, add=atomic_add)
    cuda.to_device = to_device
    cuda.device_array = device_array
    cuda.synchronize = lambda: None
    return numba


def loop_main(ref_root: str, iters: int = 1000):
    """Run the host loop of rastrigin50.py (reduced by LOOP_SUBS) to its end (or
    `iters` expansions) and record, per iteration: the UB after the sampling
    kernel, the survivors ruleOutGPU appended, the list length after the update,
    and the entry selected as the next parent (its iteration, child position,
    cycle and box); at the end, the printed enclosure and output regions.
    Written to reference_loop_rastrigin10.npz.  Every child's interval
    operations run as Python with exact rational rounding: about a minute per
    iteration."""
    oracle.build()
    path = os.path.join(ref_root, LOOP_SCRIPT)
    src = open(path).read()
    for old, new, count in LOOP_SUBS:
        if src.count(old) != count:
            raise SystemExit(f"{LOOP_SCRIPT}: expected {count} x {old!r}, found {src.count(old)}")
        src = src.replace(old, new)
    sys.modules["numba"] = make_kernel_runtime()
    sys.modules["IARastrigin"] = load_updated_ia(ref_root, False)
    rec = {"ub": [], "n_surv": [], "pool": [], "sel_iter": [], "sel_pos": [], "sel_cyc": [], "parent": []}
    t0 = time.time()
    ns: dict = {"__name__": "ref_loop"}

    def hook(*a, **k):
        msg = " ".join(str(x) for x in a)
        if msg.startswith("Number of remaining regions"):
            rec["ub"].append(float(ns["lowestUpperVal"]))
            rec["n_surv"].append(int(ns["length"]))
            rec["pool"].append(int(ns["lengthList"]))
            print(f"iteration {len(rec['ub']) - 1}: UB {rec['ub'][-1]!r}, survivors {rec['n_surv'][-1]}, "
                  f"list {rec['pool'][-1]}, {time.time() - t0:.0f} s", flush=True)
        elif msg.startswith("The selected region for the next iteration step is"):
            rec["sel_iter"].append(int(ns["iteration"]))
            rec["sel_pos"].append(int(ns["index"]))
            rec["sel_cyc"].append(int(ns["cycleIdxVal"]))
            rec["parent"].append(np.array(ns["selected_region"], dtype=np.float64))
            if len(rec["sel_iter"]) >= iters:
                raise _LoopDone()
    ns["print"] = hook
    finished = True
    try:
        exec(compile(src, path, "exec"), ns)
    except _LoopDone:
        finished = False
    out = {k: np.array(v) for k, v in rec.items()}
    out["n"] = np.array([LOOP_N]); out["wid"] = np.array([LOOP_WID])
    out["finished"] = np.array([int(finished)])
    if finished:
        # what the script prints at the end: the enclosure, the output regions, the iterations
        out["lb"] = np.array([float(np.min(ns["outputValLower"]))])
        out["ub_final"] = np.array([float(np.min(ns["outputValUpper"]))])
        out["output"] = np.array(ns["output"], dtype=np.float64)
        out["output_lb"] = np.array(ns["outputValLower"], dtype=np.float64)
        out["iterations"] = np.array([int(ns["iter"])])
    dst = os.path.join(HERE, "reference_loop_rastrigin10.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, len(rec["ub"]), "iterations", "(finished)" if finished else "(stopped)")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else "/root/reference"
    if "--loop" in sys.argv:
        loop_main(root, int(args[1]) if len(args) > 1 else 1000)
    elif "--codelist" in sys.argv:
        codelist_main(root, args[1:] or None)
    elif "--levy10000" in sys.argv:
        levy10000_main(root)
    elif "--codelist-large" in sys.argv:
        codelist_large_main(root)
    elif "--large" in sys.argv:
        large_main(root)
    else:
        main(root)
