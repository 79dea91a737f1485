"""GPU path (libgpugo.so through its C ABI) against the CPU oracle.

Integer work must match bit for bit: the survivor count per iteration, the
list length, the selected parent per iteration and the UB sequence.  Every
bound is produced by the same operation sequence on both sides, so lower
bounds, sampled upper bounds and final enclosures are compared exactly too.
"""
import os
from types import SimpleNamespace as NS

import numpy as np
import pytest

import gpugo_gb300 as G
from gpugo_gb300 import problems as P

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from gpugo_gb300 import build
    build.build()
    sm, nsm = G.device_info()
    assert sm >= 100, f"unexpected device sm_{sm}"


def _same(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return a.shape == b.shape and np.all((a == b) | (np.isnan(a) & np.isnan(b)))


def _ref_problem(g, name):
    return P.Problem(int(g[name + "_family"][0]), 50, g[name + "_domain"], g[name + "_coef"], wid=4, group=10,
                     samples=10, stop_mode=P.STOP_WIDTH, width_tol=1e-4, ub_init=1e6)


@pytest.mark.parametrize("name", ["rastrigin", "rosenbrock", "ackley", "griewank"])
def test_children_reference_setups(oracle_lib, name):
    """50-variable reference scripts (wid 4, cycles of 10): per-child bounds and flags."""
    g = np.load(GOLD)
    p = _ref_problem(g, name)
    rng = np.random.default_rng(3)
    for k, cyc in enumerate([1, 11, 41]):
        pbox = g[name + "_parents"][k]
        codes = np.concatenate([rng.integers(0, 4 ** 10, 3000), [0, 4 ** 10 - 1]]).astype(np.uint64)
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, cyc, codes, 1e300)
        ub = float(np.quantile(lb_o, 0.5))
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, cyc, codes, ub)
        lb_g, s_g, f_g = G.eval_children(p, pbox, cyc, codes, ub)
        assert _same(lb_g, lb_o), name
        assert _same(s_g, s_o), name
        assert _same(f_g, f_o), name


GOLD_1000 = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors_1000.npz")


@pytest.mark.parametrize("name", ["rastrigin", "rosenbrock", "ackley", "griewank"])
def test_children_reference_1000_variable_scripts(oracle_lib, name):
    """The reference's 1000-variable scripts (rastrigin1000.py, ...): the term
    tables no longer fit shared memory, so the children are bounded from the
    global copy.  GPU against the oracle on random codes under each golden
    parent, and against the reference's own values on the golden codes."""
    g = np.load(GOLD_1000)
    p = P.Problem(int(g[name + "_family"][0]), 1000, g[name + "_domain"], g[name + "_coef"], wid=4, group=10,
                  samples=10, stop_mode=P.STOP_WIDTH, width_tol=1e-4, ub_init=1e6)
    rng = np.random.default_rng(5)
    cycs, pidx, gcode = g[name + "_cyc"], g[name + "_parent_idx"], g[name + "_code"]
    for k, pbox in enumerate(g[name + "_parents"]):
        cyc = int(cycs[pidx == k][0])
        mine = gcode[pidx == k].astype(np.uint64)
        codes = np.concatenate([rng.integers(0, 4 ** 10, 600).astype(np.uint64), mine])
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, cyc, codes, 1e300)
        ub = float(np.quantile(lb_o, 0.5))
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, cyc, codes, ub)
        lb_g, s_g, f_g = G.eval_children(p, pbox, cyc, codes, ub)
        assert _same(lb_g, lb_o) and _same(s_g, s_o) and _same(f_g, f_o), name
        lb_r, s_r = g[name + "_lb"][pidx == k], g[name + "_samp"][pidx == k]
        lb_m, s_m = lb_g[-mine.size:], s_g[-mine.size:]
        if name in ("rastrigin", "rosenbrock"):
            assert _same(lb_m, lb_r) and _same(s_m, s_r), name
        else:
            assert np.all(lb_m <= lb_r) and np.all(s_m >= s_r), name


CFGS = [
    ("cfg1", lambda: P.config1()),
    ("cfg2", lambda: P.config2()),
    ("expsqrt5", lambda: P.instance(P.EXPSQRT, 5, 11, 1e-6)),
    ("prodcos4", lambda: P.instance(P.PRODCOS, 4, 12, 1e-6)),
    ("cosquad7", lambda: P.instance(P.COSQUAD, 7, 13, 1e-6)),
    ("chained3", lambda: P.instance(P.CHAINED, 3, 14, 1e-6)),
    ("expsqrt12", lambda: P.instance(P.EXPSQRT, 12, 15, 1e-4)),
    ("prodcos10", lambda: P.instance(P.PRODCOS, 10, 16, 1e-6)),
]


@pytest.mark.parametrize("name,make", CFGS, ids=[c[0] for c in CFGS])
def test_children_baseline_families(oracle_lib, name, make):
    p = make()
    rng = np.random.default_rng(4)
    pbox = p.domain.copy()
    M = p.children_per_iter
    codes = np.unique(np.concatenate([rng.integers(0, M, 4000), [0, M - 1]])).astype(np.uint64)
    for cyc in sorted({1, 1 + p.group * ((p.n - 1) // p.group)}):
        Mc = p.wid ** min(p.group, p.n - cyc + 1)
        cc = codes[codes < Mc]
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, cyc, cc, 1e300)
        ub = float(np.quantile(lb_o, 0.3))
        lb_o, s_o, f_o, _ = oracle_lib.eval_children(p, pbox, cyc, cc, ub)
        lb_g, s_g, f_g = G.eval_children(p, pbox, cyc, cc, ub)
        assert _same(lb_g, lb_o) and _same(s_g, s_o) and _same(f_g, f_o)


def _compare_solves(p, oracle_lib, box_cap=4096):
    ro = oracle_lib.solve(p, box_cap=box_cap, trace_cap=100000)
    rg = G.solve(p, box_cap=box_cap, trace_cap=100000)
    assert rg.iterations == ro.iterations
    for k in ("ub", "n_surv", "pool", "sel"):
        assert _same(rg.trace[k], ro.trace[k]), k
    assert rg.lb == ro.lb and rg.ub == ro.ub
    assert rg.pool_size == ro.pool_size and rg.n_boxes == ro.n_boxes
    assert _same(rg.boxes.reshape(rg.boxes.shape[0], 2 * p.n), ro.boxes.reshape(ro.boxes.shape[0], 2 * p.n))
    assert _same(rg.box_lbs, ro.box_lbs)
    return rg, ro


@pytest.mark.parametrize("name,make", CFGS[:6], ids=[c[0] for c in CFGS[:6]])
def test_solve_trace_parity(oracle_lib, name, make):
    p = make()
    p.max_iter = 3000
    rg, ro = _compare_solves(p, oracle_lib)
    assert rg.status == G.CERTIFIED and ro.status == 0
    assert rg.lb <= 0.0 <= rg.ub and rg.ub - rg.lb <= p.gap_tol
    # the minimiser point achieves the UB: a plain FP64 evaluation lies in the enclosure
    assert rg.xhat is not None
    fx = p.evaluate(rg.xhat)
    assert rg.lb - 1e-12 <= fx <= rg.ub + 1e-12


def test_solve_matches_the_reference_host_loop(oracle_lib):
    """The whole solve against the reference's own top-level loop
    (tests/golden/reference_loop_rastrigin10.npz: rastrigin50.py reduced to 10
    variables, 1024 children per iteration, run to its end): every iteration's
    UB, survivors, list length and selected parent, and the printed enclosure
    and output region, on the GPU and in the oracle."""
    from test_oracle_golden import LOOP, check_loop_trace, loop_problem
    g = np.load(LOOP)
    p = loop_problem(g)
    rg, ro = _compare_solves(p, oracle_lib, box_cap=64)
    check_loop_trace(rg, g)


def test_solve_large_list_parity(oracle_lib):
    """Lists of tens of thousands of entries take the grid-wide compaction and
    argmin path instead of the block-level one; the trace must not change."""
    p = P.instance(P.COSQUAD, 32, 20, 1e-6)
    p.max_iter = 3000
    rg, ro = _compare_solves(p, oracle_lib, box_cap=64)
    assert rg.status == G.CERTIFIED and max(ro.trace["pool"]) > 4096


def test_solve_width_mode_parity(oracle_lib):
    p = P.instance(P.COSQUAD, 4, 99, tol=0.0, split=(4, 2))
    p.stop_mode = P.STOP_WIDTH
    p.width_tol = 1e-3
    p.ub_init = 1e6
    rg, ro = _compare_solves(p, oracle_lib)
    assert rg.status == G.FINISHED and rg.n_boxes >= 1


def test_solve_reference_rastrigin_iterations(oracle_lib):
    """The 50-variable Rastrigin script's loop (4^10 children per iteration), 4 iterations."""
    g = np.load(GOLD)
    p = _ref_problem(g, "rastrigin")
    p.max_iter = 4
    rg, ro = _compare_solves(p, oracle_lib, box_cap=16)
    assert rg.status == G.ITER_LIMIT and rg.boxes_bounded == 4 * 4 ** 10


def test_engine_batch_matches_single(oracle_lib):
    """Each result is the same alone and in a mixed batch."""
    probs = [make() for _, make in CFGS] + P.config4(count=24, seed=77, nmax=12)
    for p in probs:
        p.max_iter = 2000
    singles = [G.solve(p, box_cap=8, trace_cap=4096) for p in probs]
    with G.Engine(max_slots=16, arena_bytes=2 << 30) as eng:
        batch = eng.solve_all(probs, box_cap=8)
    for p, a, b in zip(probs, singles, batch):
        assert (a.lb, a.ub, a.iterations, a.status, a.pool_size) == (b.lb, b.ub, b.iterations, b.status, b.pool_size), p.tag
        assert _same(a.boxes, b.boxes)


def _results_equal(a, b):
    """Equal results.  The count of evaluated samples is not compared: candidates
    are filtered against the running UB, which depends on the order in which the
    batch's warps reach them (the results do not)."""
    assert (a.lb, a.ub, a.iterations, a.status, a.pool_size, a.n_boxes, a.boxes_bounded) == \
        (b.lb, b.ub, b.iterations, b.status, b.pool_size, b.n_boxes, b.boxes_bounded)
    assert _same(a.boxes, b.boxes) and _same(a.box_lbs, b.box_lbs)
    assert (a.xhat is None) == (b.xhat is None)
    if a.xhat is not None:
        assert _same(a.xhat, b.xhat)


@pytest.mark.parametrize("cap", [0, 1, 4])
def test_batch_admission_matches_single_submits(cap):
    """gpugo_submit_batch: one call admits what as many gpugo_submit calls would,
    each problem's outputs land in its part of the packed buffers, and a full
    engine admits a prefix (the rest follow once slots are free)."""
    probs = [make() for _, make in CFGS] + P.config4(count=10, seed=5, nmax=12)
    for p in probs:
        p.max_iter = 2000
    with G.Engine(max_slots=len(probs), arena_bytes=2 << 30) as eng:
        ts = [eng.submit(p, box_cap=cap) for p in probs]
        eng.run(0)
        one = dict(eng.poll())
    with G.Engine(max_slots=5, arena_bytes=2 << 30) as eng:
        many, nxt = {}, 0
        while nxt < len(probs):
            got = eng.submit_many(probs[nxt:], box_cap=cap)
            assert len(got) == min(5, len(probs) - nxt)
            for t in got:
                many[t] = nxt
                nxt += 1
            eng.run(0)
            done = dict(eng.poll())
            assert sorted(done) == sorted(got)
            for t, r in done.items():
                _results_equal(one[ts[many[t]]], r)


def test_batch_admission_stops_at_an_invalid_spec():
    """An invalid description ends the batch with its error; those before it are
    admitted and solve."""
    good = [make() for _, make in CFGS]
    bad = P.instance(P.COSQUAD, 6, 3, 1e-6)
    bad.wid = 1                                    # the library refuses wid < 2
    with G.Engine(max_slots=8, arena_bytes=1 << 30) as eng:
        with pytest.raises(G.GpugoError) as e:
            eng.submit_many(good[:2] + [bad] + good[2:], box_cap=2)
        assert e.value.code == G._lib.ERR_INVALID and len(e.value.admitted) == 2
        eng.run(0)
        done = eng.poll()
    assert sorted(t for t, _ in done) == sorted(e.value.admitted) and all(r.certified for _, r in done)


WIDE = [
    ("cosquad40", lambda: P.instance(P.COSQUAD, 40, 21, 1e-6)),
    ("chained30", lambda: P.instance(P.CHAINED, 30, 22, 1e-6)),
    ("expsqrt20", lambda: P.instance(P.EXPSQRT, 20, 18, 1e-6)),
    ("expsqrt32", lambda: P.instance(P.EXPSQRT, 32, 17, 1e-4)),
    ("prodcos24", lambda: P.instance(P.PRODCOS, 24, 19, 1e-6)),
]


@pytest.mark.parametrize("name,make", WIDE, ids=[c[0] for c in WIDE])
def test_solve_trace_parity_wide(oracle_lib, name, make):
    """Split groups that cycle through the coordinates (n > group)."""
    p = make()
    p.max_iter = 3000
    rg, ro = _compare_solves(p, oracle_lib, box_cap=64)
    assert rg.status == G.CERTIFIED


@pytest.mark.parametrize("mode", [G._lib.CAND_WARP, G._lib.CAND_LANE], ids=["warp", "lane"])
def test_engine_batch_matches_oracle(oracle_lib, mode):
    """A batch in each candidate scheduling mode against the oracle, trace for trace."""
    probs = [make() for _, make in WIDE + CFGS]
    for p in probs:
        p.max_iter = 3000
    ros = [oracle_lib.solve(p, box_cap=16, trace_cap=100000) for p in probs]
    with G.Engine(max_slots=len(probs), arena_bytes=4 << 30, cand_mode=mode) as eng:
        tickets = [eng.submit(p, box_cap=16, trace_cap=100000) for p in probs]
        eng.run(0)
        done = dict(eng.poll())
    for t, p, ro in zip(tickets, probs, ros):
        rg = done[t]
        assert (rg.iterations, rg.lb, rg.ub, rg.pool_size) == (ro.iterations, ro.lb, ro.ub, ro.pool_size), p.tag
        for k in ("ub", "n_surv", "pool", "sel"):
            assert _same(rg.trace[k], ro.trace[k]), (p.tag, k)
        assert _same(rg.box_lbs, ro.box_lbs), p.tag


def test_iteration_streamed_in_passes(oracle_lib):
    """The shape of config 3 scaled down: the exp-sqrt composite at n = 16 split
    in 2 parts per coordinate (2^16 children per iteration, every first-level
    child touching the minimiser at the centre of the domain), solved in one
    children pass per iteration and in passes of 4096 and of 1000 children
    (the candidate queue refilled 16 and 66 times per iteration): every trace
    equals the oracle's."""
    p = P.instance(P.EXPSQRT, 16, 7, 1e-4, split=(2, 16))
    p.max_iter = 4
    ro = oracle_lib.solve(p, box_cap=16, trace_cap=64)
    assert ro.trace["n_surv"][0] == 1 << 16          # nothing of the first split can be ruled out
    for chunk in (0, 4096, 1000):
        with G.Engine(max_slots=1, arena_bytes=1 << 30, chunk_children=chunk) as eng:
            eng.submit(p, box_cap=16, trace_cap=64)
            eng.run(0)
            (_, rg), = eng.poll()
        assert (rg.iterations, rg.lb, rg.ub, rg.pool_size, rg.status) == \
            (ro.iterations, ro.lb, ro.ub, ro.pool_size, G.ITER_LIMIT), chunk
        for k in ("ub", "n_surv", "pool", "sel"):
            assert _same(rg.trace[k], ro.trace[k]), (chunk, k)
        assert _same(rg.box_lbs, ro.box_lbs), chunk


def test_batch_streamed_in_passes(oracle_lib):
    """A mixed batch whose children passes end inside instances: instances are
    updated only after the iteration's last pass, and every result equals the
    oracle's."""
    probs = [make() for _, make in CFGS[:4]] + P.config4(count=10, seed=78, nmax=10)
    for p in probs:
        p.max_iter = 3000
    ros = [oracle_lib.solve(p, box_cap=8, trace_cap=100000) for p in probs]
    with G.Engine(max_slots=len(probs), arena_bytes=2 << 30, chunk_children=777) as eng:
        tickets = [eng.submit(p, box_cap=8, trace_cap=100000) for p in probs]
        eng.run(0)
        done = dict(eng.poll())
    for t, p, ro in zip(tickets, probs, ros):
        rg = done[t]
        assert (rg.iterations, rg.lb, rg.ub, rg.pool_size) == (ro.iterations, ro.lb, ro.ub, ro.pool_size), p.tag
        for k in ("ub", "n_surv", "pool", "sel"):
            assert _same(rg.trace[k], ro.trace[k]), (p.tag, k)


EDGE = [
    ("cosquad1", lambda: P.instance(P.COSQUAD, 1, 31, 1e-6)),
    ("chained2_s1", lambda: P.instance(P.CHAINED, 2, 32, 1e-6, samples=1)),
    ("expsqrt6_s20", lambda: P.instance(P.EXPSQRT, 6, 33, 1e-5, samples=20)),
    ("expsqrt9_s14", lambda: P.instance(P.EXPSQRT, 9, 34, 1e-5, samples=14)),
    ("prodcos5_s40", lambda: P.instance(P.PRODCOS, 5, 35, 1e-6, samples=40)),
    ("cosquad3_w9", lambda: P.instance(P.COSQUAD, 3, 36, 1e-6, split=(9, 3), samples=3)),
    # lane groups of S lanes for short candidate queues: 4, 2 and 2 groups a warp
    # with idle lanes above them, then the first S that takes a warp per candidate
    ("chained6_s7", lambda: P.instance(P.CHAINED, 6, 37, 1e-6, samples=7)),
    ("prodcos6_s12", lambda: P.instance(P.PRODCOS, 6, 38, 1e-6, samples=12)),
    ("cosquad5_s16", lambda: P.instance(P.COSQUAD, 5, 39, 1e-6, samples=16)),
    ("chained4_s17", lambda: P.instance(P.CHAINED, 4, 40, 1e-6, samples=17)),
]


@pytest.mark.parametrize("name,make", EDGE, ids=[c[0] for c in EDGE])
def test_solve_trace_parity_edge_shapes(oracle_lib, name, make):
    """One variable, one sample point, more sample points than lanes, the largest
    sample count the warp-wide exp-sqrt path takes and the first it does not."""
    p = make()
    p.max_iter = 3000
    rg, ro = _compare_solves(p, oracle_lib, box_cap=16)
    assert rg.status == G.CERTIFIED


def test_lane_groups_of_mixed_sizes_in_one_batch(oracle_lib):
    """Short queues with candidates of instances of different S side by side:
    each round takes entries of one group size, the others wait for their own
    rounds; every solve matches the oracle trace for trace."""
    probs = [P.instance(fam, n, 60 + k, 1e-6, samples=S)
             for k, (fam, n, S) in enumerate([(P.CHAINED, 5, 7), (P.CHAINED, 5, 10), (P.COSQUAD, 4, 12),
                                               (P.PRODCOS, 4, 16), (P.CHAINED, 3, 17), (P.COSQUAD, 6, 1),
                                               (P.EXPSQRT, 4, 10)])]
    for p in probs:
        p.max_iter = 3000
    ros = [oracle_lib.solve(p, box_cap=8, trace_cap=100000) for p in probs]
    with G.Engine(max_slots=len(probs), arena_bytes=2 << 30, cand_mode=G._lib.CAND_WARP) as eng:
        tickets = [eng.submit(p, box_cap=8, trace_cap=100000) for p in probs]
        eng.run(0)
        done = dict(eng.poll())
    for t, p, ro in zip(tickets, probs, ros):
        rg = done[t]
        assert (rg.iterations, rg.lb, rg.ub, rg.pool_size) == (ro.iterations, ro.lb, ro.ub, ro.pool_size), p.tag
        for k in ("ub", "n_surv", "pool", "sel"):
            assert _same(rg.trace[k], ro.trace[k]), (p.tag, k)


def test_finalized_results_match_collected():
    """Results of small outputs are assembled on the device (finalize_kernel);
    the host path (taken with a trace) gives the same bits."""
    probs = [make() for _, make in CFGS + WIDE]
    w = P.instance(P.COSQUAD, 4, 99, tol=0.0, split=(4, 2))
    w.stop_mode = P.STOP_WIDTH
    w.width_tol = 1e-3
    w.ub_init = 1e6
    probs.append(w)
    for p in probs:
        p.max_iter = 3000
    for cap in (1, 16):
        for p in probs:
            x = G.solve(p, box_cap=cap, trace_cap=100000)   # host path
            y = G.solve(p, box_cap=cap)                     # device records
            assert (x.lb, x.ub, x.iterations, x.status, x.pool_size, x.n_boxes) == \
                (y.lb, y.ub, y.iterations, y.status, y.pool_size, y.n_boxes), p.tag
            assert _same(x.boxes, y.boxes) and _same(x.box_lbs, y.box_lbs), p.tag
            assert (x.xhat is None) == (y.xhat is None), p.tag
            if x.xhat is not None:
                assert _same(x.xhat, y.xhat), p.tag


def test_pool_overflow_reports_error():
    """Host-side fault injection: a pool too small for the survivors."""
    p = P.config2()
    p.pool_cap = 4
    with pytest.raises(G.GpugoError) as e:
        G.solve(p)
    assert e.value.code == -4
    # the library stays usable afterwards
    r = G.solve(P.config1())
    assert r.certified


def test_parent_overflow_reports_error():
    p = P.config2()
    p.parent_cap = 3
    with pytest.raises(G.GpugoError) as e:
        G.solve(p)
    assert e.value.code == -5


def test_bounded_wait_expires_cleanly():
    """A device wait budget of ~zero makes every grid barrier give up: the run
    returns GPUGO_ERR_TIMEOUT and the context stays usable."""
    with G.Engine(max_slots=2, arena_bytes=256 << 20, wait_timeout_s=1e-9) as eng:
        eng.submit(P.config2())
        with pytest.raises(G.GpugoError) as e:
            eng.run()
        assert e.value.code == -6
    r = G.solve(P.config1())
    assert r.certified


def _levy12_codelist():
    from gpugo_gb300 import objectives as O
    return O.problem("levy", 12, tol=1e-6)


CKPT = [
    ("cfg2", lambda: P.config2()),
    ("expsqrt20", lambda: P.instance(P.EXPSQRT, 20, 18, 1e-6)),
    ("chained30", lambda: P.instance(P.CHAINED, 30, 22, 1e-6)),
    ("levy12_codelist", _levy12_codelist),
]


@pytest.mark.parametrize("name,make", CKPT, ids=[c[0] for c in CKPT])
def test_checkpoint_resume_is_bit_identical(oracle_lib, name, make):
    """A solve checkpointed after three iterations and restored into another engine
    (next to another solve) ends exactly like the uninterrupted solve and the oracle."""
    p = make()
    p.max_iter = 3000
    ro = oracle_lib.solve(p, box_cap=16, trace_cap=100000)
    with G.Engine(max_slots=4, arena_bytes=2 << 30) as e1:
        t = e1.submit(p, box_cap=16, trace_cap=100000)
        e1.run(3)
        data = e1.checkpoint(t)
        e1.run(0)
        (_, a), = e1.poll()
    with G.Engine(max_slots=4, arena_bytes=2 << 30) as e2:
        e2.submit(P.config1(), box_cap=4)
        t2 = e2.restore(p, data, box_cap=16, trace_cap=100000)
        e2.run(0)
        done = dict(e2.poll())
    b = done[t2]
    for x in (a, b):
        assert (x.iterations, x.lb, x.ub, x.status, x.pool_size, x.n_boxes) == \
            (ro.iterations, ro.lb, ro.ub, G.CERTIFIED, ro.pool_size, ro.n_boxes)
        for k in ("ub", "n_surv", "pool", "sel"):
            assert _same(x.trace[k], ro.trace[k]), k
        assert _same(x.box_lbs, ro.box_lbs)
    assert _same(a.boxes, b.boxes) and a.samples_evaluated == b.samples_evaluated
    assert (a.xhat is None) == (b.xhat is None)
    if a.xhat is not None:
        assert _same(a.xhat, b.xhat)


def test_checkpoint_rejects_unadmitted_and_bad_data():
    p = P.config1()
    with G.Engine(max_slots=2, arena_bytes=1 << 30) as e:
        t = e.submit(p, box_cap=4)
        with pytest.raises(G.GpugoError) as err:
            e.checkpoint(t)                       # not run yet
        assert err.value.code == -7
        e.run(1)
        data = bytearray(e.checkpoint(t))
        assert G.checkpoint_ok(bytes(data))       # a real checkpoint passes the host checks
        data[0] ^= 0xFF                           # corrupt the magic
        assert not G.checkpoint_ok(bytes(data))
        with pytest.raises(G.GpugoError) as err:
            e.restore(p, bytes(data))
        assert err.value.code == -1
        e.run(0)
        (_, r), = e.poll()
        assert r.certified
