"""The CPU oracle against golden vectors produced by the reference's own code.

tests/golden/make_golden.py executed the reference's device functions
(rastrigin50.py, rosenbrock50.py, ackley50.py, griewank50.py with the updated
interval library) on fixed parent boxes and child codes.
"""
import os
from types import SimpleNamespace as NS

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _problem(g, name):
    return NS(family=int(g[name + "_family"][0]), n=50, wid=4, group=10, samples=10, stop_mode=0,
              width_tol=1e-4, gap_tol=0.0, ub_init=1e6, domain=g[name + "_domain"], coef=g[name + "_coef"])


def _eval(oracle_lib, g, name):
    p = _problem(g, name)
    par, pidx, cyc, code = g[name + "_parents"], g[name + "_parent_idx"], g[name + "_cyc"], g[name + "_code"]
    out = {"lb": [], "samp": [], "dflag": [], "flag_below": []}
    for k in range(code.size):
        lb, samp, flag, dflag = oracle_lib.eval_children(p, par[pidx[k]], int(cyc[k]), np.array([code[k]]), 1e300)
        out["lb"].append(lb[0]); out["samp"].append(samp[0]); out["dflag"].append(dflag[0])
        ref_lb = g[name + "_lb"][k]
        _, _, fb, _ = oracle_lib.eval_children(p, par[pidx[k]], int(cyc[k]), np.array([code[k]]),
                                               ref_lb - abs(ref_lb) * 1e-9 - 1e-300)
        out["flag_below"].append(fb[0])
    return {k: np.array(v) for k, v in out.items()}


@pytest.mark.parametrize("name", ["rastrigin", "rosenbrock"])
def test_bit_exact_families(oracle_lib, gold, name):
    """Same interval semantics as the reference: every bound identical bit for bit."""
    r = _eval(oracle_lib, gold, name)
    np.testing.assert_array_equal(r["lb"], gold[name + "_lb"])
    np.testing.assert_array_equal(r["samp"], gold[name + "_samp"])
    np.testing.assert_array_equal(r["dflag"], gold[name + "_dflag"])
    np.testing.assert_array_equal(r["flag_below"], gold[name + "_flag_below"])


@pytest.mark.parametrize("name", ["ackley", "griewank"])
def test_enclosure_families(oracle_lib, gold, name):
    """Constants the reference rounds to nearest (1/n, e, 1/sqrt(i), 1/d) are carried
    as enclosures here, so bounds may only be wider, by a few ulps."""
    r = _eval(oracle_lib, gold, name)
    ref_lb, ref_s = gold[name + "_lb"], gold[name + "_samp"]
    assert np.all(r["lb"] <= ref_lb)
    assert np.all(r["samp"] >= ref_s)
    np.testing.assert_allclose(r["lb"], ref_lb, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(r["samp"], ref_s, rtol=1e-13, atol=1e-13)
    m = gold[name + "_dflag"] >= 0
    np.testing.assert_array_equal(r["dflag"][m], gold[name + "_dflag"][m])


def test_box_decoder(oracle_lib, gold):
    """completeRegion / selectVarInSubRegion (ackley50.py:482-594, :820-948)."""
    p = _problem(gold, "rastrigin")
    for t in range(gold["decoder_code"].size):
        pb = gold["rastrigin_parents"][gold["decoder_parent_idx"][t]]
        box = oracle_lib.child_box(p, pb, int(gold["decoder_cyc"][t]), int(gold["decoder_code"][t]))
        np.testing.assert_array_equal(box, gold["decoder_complete"][t])
        np.testing.assert_array_equal(box, gold["decoder_select"][t])


GOLD_1000 = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors_1000.npz")


def _eval_n(oracle_lib, g, name, n):
    p = NS(family=int(g[name + "_family"][0]), n=n, wid=4, group=10, samples=10, stop_mode=0, width_tol=1e-4,
           gap_tol=0.0, ub_init=1e6, domain=g[name + "_domain"], coef=g[name + "_coef"])
    par, pidx, cyc, code = g[name + "_parents"], g[name + "_parent_idx"], g[name + "_cyc"], g[name + "_code"]
    lbs, samps, dflags = [], [], []
    for k in range(code.size):
        lb, samp, _, dflag = oracle_lib.eval_children(p, par[pidx[k]], int(cyc[k]), np.array([code[k]]), 1e300)
        lbs.append(lb[0]); samps.append(samp[0]); dflags.append(dflag[0])
    return np.array(lbs), np.array(samps), np.array(dflags)


@pytest.mark.parametrize("name", ["rastrigin", "rosenbrock", "ackley", "griewank"])
def test_reference_1000_variable_scripts(oracle_lib, name):
    """The same families at the reference's 1000-variable scripts (rastrigin1000.py,
    ...): bit for bit where the reference's constants are exact, otherwise the
    enclosure rule of the 50-variable vectors."""
    g = np.load(GOLD_1000)
    lb, samp, dflag = _eval_n(oracle_lib, g, name, 1000)
    ref_lb, ref_s, ref_d = g[name + "_lb"], g[name + "_samp"], g[name + "_dflag"]
    if name in ("rastrigin", "rosenbrock"):
        np.testing.assert_array_equal(lb, ref_lb)
        np.testing.assert_array_equal(samp, ref_s)
    else:
        assert np.all(lb <= ref_lb) and np.all(samp >= ref_s)
        np.testing.assert_allclose(lb, ref_lb, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(samp, ref_s, rtol=1e-12, atol=1e-12)
    m = ref_d >= 0
    np.testing.assert_array_equal(dflag[m], ref_d[m])


LOOP = os.path.join(os.path.dirname(__file__), "golden", "reference_loop_rastrigin10.npz")


def loop_problem(g):
    """The problem the reference's host loop solved for reference_loop_rastrigin10.npz:
    rastrigin50.py reduced to 10 variables split in 2 parts each (one cycle of
    10, 1024 children per iteration), its own domain, width rule 1e-4, initial
    UB 1e6 and 10 samples (tests/golden/make_golden.py, LOOP_SUBS)."""
    from gpugo_gb300 import problems as P
    n, wid = int(g["n"][0]), int(g["wid"][0])
    return P.Problem(P.COSQUAD, n, np.tile([-5.5, 6.0], n),
                     np.concatenate([np.ones(n), np.full(n, 10.0), np.ones(n)]), wid=wid, group=10, samples=10,
                     stop_mode=P.STOP_WIDTH, width_tol=1e-4, ub_init=1e6)


def check_loop_trace(r, g):
    """A solve's per-iteration trace and result against the reference's own host
    loop (ackley50.py:1269-1370 in its Rastrigin form): the UB after each
    sampling kernel, the survivors ruleOutGPU appended, the list length, the
    entry selected as the next parent (its iteration and child position, whose
    tie-break the reference's atomics give in thread order), and at the end the
    printed enclosure, output regions and iteration count."""
    assert g["finished"][0] == 1
    assert r.iterations == g["iterations"][0]
    np.testing.assert_array_equal(r.trace["ub"], g["ub"])
    np.testing.assert_array_equal(r.trace["n_surv"], g["n_surv"])
    np.testing.assert_array_equal(r.trace["pool"], g["pool"])
    assert np.all(g["sel_cyc"] == 1)                 # one cycle: every parent starts at coordinate 1
    want = (g["sel_iter"].astype(np.int64) << 32) | g["sel_pos"].astype(np.int64)
    np.testing.assert_array_equal(r.trace["sel"][:want.size], want)
    assert np.all(r.trace["sel"][want.size:] == -1)
    assert r.lb == g["lb"][0] and r.ub == g["ub_final"][0]
    boxes = np.asarray(r.boxes).reshape(-1, 2 * int(g["n"][0]))
    np.testing.assert_array_equal(boxes, g["output"])
    np.testing.assert_array_equal(r.box_lbs, g["output_lb"])


def test_oracle_reproduces_the_reference_host_loop(oracle_lib):
    """The reference's own top-level loop (rastrigin50.py:844-1302, run by
    make_golden.py --loop with its kernels executed thread by thread) pins the
    oracle's selection, cycle, width-rule and UB bookkeeping, not only its
    per-child bounds."""
    g = np.load(LOOP)
    r = oracle_lib.solve(loop_problem(g), box_cap=64, trace_cap=1000, skip_samples=False)
    check_loop_trace(r, g)
    r2 = oracle_lib.solve(loop_problem(g), box_cap=64, trace_cap=1000, skip_samples=True)
    check_loop_trace(r2, g)
