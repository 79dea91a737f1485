"""Code-list objectives on the GPU (libgpugo.so's interpreter) against the
oracle's interpreter and the reference's own code lists, bit for bit."""
import os

import numpy as np
import pytest

import gpugo_gb300 as G
from gpugo_gb300 import codelist as CL
from gpugo_gb300 import objectives as O
from gpugo_gb300 import problems as P

pytestmark = pytest.mark.gpu

CL_GOLD = os.path.join(os.path.dirname(__file__), "golden", "codelist_vectors.npz")
NOT_REPRODUCED = {("deflected", "dflag"), ("cosine", "samp")}


@pytest.fixture(scope="module", autouse=True)
def built():
    from gpugo_gb300 import build
    build.build()
    sm, _ = G.device_info()
    assert sm >= 100


def _same(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("name", sorted(O.REFERENCE))
def test_children_match_reference_code_lists(oracle_lib, name):
    """50 variables, wid 4, cycles of 10 (the reference scripts' setup)."""
    z = np.load(CL_GOLD)
    f, g, _ = O.REFERENCE[name](50)
    p = P.Problem(P.CODELIST, 50, z[name + "_domain"], CL.compile_objective(f, 50, g).coef, wid=4, group=10,
                  samples=10)
    rng = np.random.default_rng(5)
    pidx, cyc = z[name + "_parent_idx"], z[name + "_cyc"]
    for k, pbox in enumerate(z[name + "_parents"]):
        sel = pidx == k
        cy = int(cyc[sel][0])
        gold_codes = z[name + "_code"][sel].astype(np.uint64)
        lb_g, s_g, f_g = G.eval_children(p, pbox, cy, gold_codes, 1e300)
        assert _same(lb_g, z[name + "_lb"][sel])
        if (name, "samp") not in NOT_REPRODUCED:
            assert _same(s_g, z[name + "_samp"][sel])
        if (name, "dflag") not in NOT_REPRODUCED:
            assert np.array_equal(f_g, z[name + "_dflag"][sel])
        # many more children against the oracle, with a UB that rules some out
        codes = np.concatenate([rng.integers(0, 4 ** 10, 2000), [0, 4 ** 10 - 1]]).astype(np.uint64)
        lb_o, _, _, _ = oracle_lib.eval_children(p, pbox, cy, codes, 1e300)
        ub = float(np.quantile(lb_o, 0.5))
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, cy, codes, ub)
        lb_g, s_g, f_g = G.eval_children(p, pbox, cy, codes, ub)
        assert _same(lb_g, lb_o) and _same(s_g, s_o) and np.array_equal(f_g, f_o)


def _compare(p, oracle_lib, box_cap=64):
    ro = oracle_lib.solve(p, box_cap=box_cap, trace_cap=100000)
    rg = G.solve(p, box_cap=box_cap, trace_cap=100000)
    assert rg.iterations == ro.iterations
    for k in ("ub", "n_surv", "pool", "sel"):
        assert _same(rg.trace[k], ro.trace[k]), k
    assert rg.lb == ro.lb and rg.ub == ro.ub and rg.n_boxes == ro.n_boxes
    assert _same(rg.box_lbs, ro.box_lbs)
    return rg, ro


SOLVES = [(name, n) for name in sorted(O.REFERENCE) for n in (3, 6)] + [("levy", 12), ("salomon", 10),
                                                                       ("sinusoidal", 8), ("corrupted", 9)]


@pytest.mark.parametrize("name,n", SOLVES, ids=[f"{a}{b}" for a, b in SOLVES])
def test_solve_trace_parity(oracle_lib, name, n):
    p = O.problem(name, n, tol=1e-6)
    p.max_iter = 3000
    rg, ro = _compare(p, oracle_lib)
    assert rg.status == G.CERTIFIED
    assert rg.xhat is not None
    fx = p.evaluate(rg.xhat)
    assert rg.lb - 1e-9 <= fx <= rg.ub + 1e-9


@pytest.mark.parametrize("family,n,split", [(P.CHAINED, 8, (4, 8)), (P.COSQUAD, 7, None), (P.EXPSQRT, 6, None),
                                            (P.PRODCOS, 10, None), (P.CHAINED, 20, None)])
def test_builtin_as_code_list_same_solve(family, n, split):
    """A built-in family and its code-list restatement give the same solve
    (config 2's chained quartic is the first case)."""
    p = P.instance(family, n, 200 + n, 1e-6, split)
    q = O.as_codelist(p)
    a = G.solve(p, box_cap=16, trace_cap=100000)
    b = G.solve(q, box_cap=16, trace_cap=100000)
    assert (a.lb, a.ub, a.iterations, a.pool_size) == (b.lb, b.ub, b.iterations, b.pool_size)
    for k in a.trace:
        assert _same(a.trace[k], b.trace[k]), k
    print(f"\n{p.tag}: built-in {a.device_ms:.3f} ms, code list {b.device_ms:.3f} ms, {a.iterations} iterations")


@pytest.mark.parametrize("mode,big", [(G._lib.CAND_WARP, False), (G._lib.CAND_LANE, False), (G._lib.CAND_AUTO, True)],
                         ids=["warp", "lane", "grouped160"])
def test_engine_mixed_batch(oracle_lib, mode, big):
    """Code-list and built-in instances side by side in one persistent kernel
    (160 slots take the family-grouped work lists)."""
    ns = (3, 4, 5, 6, 7) if big else (4, 7)
    probs = [O.problem(name, n, tol=1e-6) for name in sorted(O.REFERENCE) for n in ns]
    probs += P.config4(count=95 if big else 12, seed=91, nmax=10)
    probs += [O.as_codelist(p) for p in P.config4(count=30 if big else 6, seed=92, nmax=10)]
    for p in probs:
        p.max_iter = 3000
    ros = [oracle_lib.solve(p, box_cap=16, trace_cap=100000) for p in probs]
    with G.Engine(max_slots=len(probs), arena_bytes=8 << 30, cand_mode=mode) as eng:
        tickets = [eng.submit(p, box_cap=16, trace_cap=100000) for p in probs]
        eng.run(0)
        done = dict(eng.poll())
    for t, p, ro in zip(tickets, probs, ros):
        rg = done[t]
        assert (rg.iterations, rg.lb, rg.ub, rg.pool_size) == (ro.iterations, ro.lb, ro.ub, ro.pool_size), p.tag
        for k in ("ub", "n_surv", "pool", "sel"):
            assert _same(rg.trace[k], ro.trace[k]), (p.tag, k)


@pytest.mark.parametrize("name,n", [("levy", 9), ("sinusoidal", 6), ("salomon", 8), ("trigonometric", 7)])
def test_term_tables_and_loops_same_solve(name, n):
    """Reductions read from term tables give the solve the loop form gives."""
    f, g, dom = O.REFERENCE[name](n)
    base = O.problem(name, n, tol=1e-6)
    loops = P.Problem(P.CODELIST, n, base.domain, CL.compile_objective(f, n, g, tables=False).coef, wid=base.wid,
                      group=base.group, samples=base.samples, gap_tol=1e-6)
    a = G.solve(base, box_cap=16, trace_cap=100000)
    b = G.solve(loops, box_cap=16, trace_cap=100000)
    assert (a.lb, a.ub, a.iterations, a.pool_size) == (b.lb, b.ub, b.iterations, b.pool_size)
    for k in a.trace:
        assert _same(a.trace[k], b.trace[k]), k
    print(f"\n{name}{n}: tables {a.device_ms:.3f} ms, loops {b.device_ms:.3f} ms, {a.iterations} iterations")


AUTO = [("levy", 7), ("sinusoidal", 6), ("salomon", 9), ("chained", 12), ("prodcos", 10)]


@pytest.mark.parametrize("name,n", AUTO, ids=[f"{a}{b}" for a, b in AUTO])
def test_auto_gradient_solve_parity(oracle_lib, name, n):
    """Gradients derived by the compiler, on the GPU against the oracle."""
    if name in O.REFERENCE:
        f, _, dom = O.REFERENCE[name](n)
        domain = np.tile(dom, n)
    else:
        fam = {"chained": P.CHAINED, "prodcos": P.PRODCOS}[name]
        base = P.instance(fam, n, 400 + n)
        f, _ = O.BUILTIN[fam](n, base.coef)
        domain = base.domain
    wid, group = P.default_split(n)
    p = P.Problem(P.CODELIST, n, domain, CL.compile_objective(f, n, "auto").coef, wid=wid, group=group, gap_tol=1e-6)
    p.max_iter = 3000
    rg, ro = _compare(p, oracle_lib)
    assert rg.status == G.CERTIFIED


def test_malformed_code_list_is_rejected():
    f, g, dom = O.levy(5)
    coef = CL.compile_objective(f, 5, g).coef.copy()
    coef.view(np.uint64)[2] = 40           # 40 registers
    p = P.Problem(P.CODELIST, 5, np.tile(dom, 5), coef, wid=3, group=5)
    with pytest.raises(G.GpugoError):
        G.solve(p)


def test_levy10000_reference_size(oracle_lib):
    """The reference's largest script (levy10000.py: 10 000 variables, wid 4,
    cycles of 10): children against the oracle at the first and the last cycle,
    then two iterations of the loop (4^10 children each)."""
    n = 10000
    f, g, dom = O.levy(n)
    p = P.Problem(P.CODELIST, n, np.tile(dom, n), CL.compile_objective(f, n, g).coef, wid=4, group=10,
                  samples=10, stop_mode=P.STOP_WIDTH, width_tol=1e-4, ub_init=1000.0)
    rng = np.random.default_rng(10)
    for cyc in (1, n - 9):
        codes = np.concatenate([rng.integers(0, 4 ** 10, 300), [0, 4 ** 10 - 1]]).astype(np.uint64)
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, p.domain, cyc, codes, 1e300)
        lb_g, s_g, f_g = G.eval_children(p, p.domain, cyc, codes, 1e300)
        assert _same(lb_g, lb_o) and _same(s_g, s_o) and np.array_equal(f_g, f_o)
    p.max_iter = 2
    r = G.solve(p, box_cap=4)
    assert r.status == G.ITER_LIMIT and r.boxes_bounded == 2 * 4 ** 10 and r.lb <= r.ub
    print(f"\nlevy10000: 2 iterations in {r.device_ms:.1f} ms, enclosure [{r.lb:.6g}, {r.ub:.6g}]")


@pytest.mark.parametrize("name", sorted(O.REFERENCE))
def test_children_match_reference_1000_variable_scripts(oracle_lib, name):
    """The seven benchmarks' 1000-variable scripts: the reference's values on
    its golden codes, and the oracle on more children with a UB that rules
    some out, at the first, a middle and the last cycle."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "codelist_vectors_1000.npz"))
    n = 1000
    f, g, _ = O.REFERENCE[name](n)
    p = P.Problem(P.CODELIST, n, z[name + "_domain"], CL.compile_objective(f, n, g).coef, wid=4, group=10,
                  samples=10)
    rng = np.random.default_rng(6)
    pidx, cyc = z[name + "_parent_idx"], z[name + "_cyc"]
    for k, pbox in enumerate(z[name + "_parents"]):
        sel = pidx == k
        cy = int(cyc[sel][0])
        lb_g, s_g, f_g = G.eval_children(p, pbox, cy, z[name + "_code"][sel].astype(np.uint64), 1e300)
        assert _same(lb_g, z[name + "_lb"][sel])
        if (name, "samp") not in NOT_REPRODUCED:
            assert _same(s_g, z[name + "_samp"][sel])
        if (name, "dflag") not in NOT_REPRODUCED:
            assert np.array_equal(f_g, z[name + "_dflag"][sel])
        codes = np.concatenate([rng.integers(0, 4 ** 10, 300), [0, 4 ** 10 - 1]]).astype(np.uint64)
        lb_o, _, _, _ = oracle_lib.eval_children(p, pbox, cy, codes, 1e300)
        ub = float(np.quantile(lb_o, 0.5))
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, cy, codes, ub)
        lb_g, s_g, f_g = G.eval_children(p, pbox, cy, codes, ub)
        assert _same(lb_g, lb_o) and _same(s_g, s_o) and np.array_equal(f_g, f_o)


@pytest.mark.parametrize("seed", range(8))
def test_random_objectives_match_oracle(oracle_lib, seed):
    """Random objectives of the front end (the generator of
    test_codelist_random: sums over one or two offsets, a fixed coordinate or an
    inner reduction inside a body, products, derived gradients): children and a
    bounded solve bit for bit against the oracle's interpreter."""
    import test_codelist_random as R
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(2, 6))
    f = R._objective(rng, n)
    p = P.Problem(P.CODELIST, n, np.tile([-2.0, 2.5], n), CL.compile_objective(f, n, "auto").coef, wid=3,
                  group=n, samples=4, max_iter=150)
    codes = np.arange(3 ** n, dtype=np.uint64)
    for t in range(3):
        w = 4.5 * 10.0 ** rng.uniform(-4, -0.3, n)
        c = rng.uniform(-2.0, 2.5 - w)
        pbox = np.empty(2 * n)
        pbox[0::2], pbox[1::2] = c, c + w
        lb_o, _, _, _ = oracle_lib.eval_children(p, pbox, 1, codes, 1e300)
        ub = float(np.quantile(lb_o, 0.5))
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, 1, codes, ub)
        lb_g, s_g, f_g = G.eval_children(p, pbox, 1, codes, ub)
        assert _same(lb_g, lb_o) and _same(s_g, s_o) and np.array_equal(f_g, f_o), (seed, t)
    _compare(p, oracle_lib)
