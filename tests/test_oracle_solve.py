"""Known answers for the CPU restatement of the B&B loop (ackley50.py:950-1396).

Every family's global minimum is 0 (at x = 0, or x = 1 for the chained family).
"""
import numpy as np
import pytest

from gpugo_gb300 import problems as P


def _check_enclosure(p, r, tol):
    assert r.lb <= 0.0 <= r.ub, (r.lb, r.ub)
    assert r.ub - r.lb <= tol
    xs = p.minimiser()
    # at least one returned box contains the analytic minimiser
    assert any(np.all((b[0::2] <= xs) & (xs <= b[1::2])) for b in r.boxes)


@pytest.mark.parametrize("make", [P.config1, P.config2])
def test_baseline_configs_certify(oracle_lib, make):
    p = make()
    r = oracle_lib.solve(p, box_cap=4096, trace_cap=4096)
    assert r.status == 0
    _check_enclosure(p, r, p.gap_tol)


@pytest.mark.parametrize("fam,n", [(P.COSQUAD, 3), (P.CHAINED, 3), (P.EXPSQRT, 2), (P.PRODCOS, 3), (P.EXPSQRT, 5)])
def test_small_families_certify(oracle_lib, fam, n):
    p = P.instance(fam, n, 1234 + n + 10 * fam, tol=1e-6)
    p.max_iter = 20000
    r = oracle_lib.solve(p, box_cap=4096)
    assert r.status == 0, r
    _check_enclosure(p, r, 1e-6)


def test_skip_samples_changes_nothing(oracle_lib):
    """Children whose LB exceeds the running UB cannot lower it: skipping their
    samples leaves the UB sequence and every decision unchanged."""
    for p in (P.config1(), P.config2(), P.instance(P.PRODCOS, 3, 5, 1e-6)):
        a = oracle_lib.solve(p, box_cap=64, trace_cap=4096, skip_samples=True)
        b = oracle_lib.solve(p, box_cap=64, trace_cap=4096, skip_samples=False)
        assert a.samples_evaluated < b.samples_evaluated
        for k in ("ub", "n_surv", "pool", "sel"):
            np.testing.assert_array_equal(a.trace[k], b.trace[k])
        assert (a.lb, a.ub, a.iterations) == (b.lb, b.ub, b.iterations)


def test_width_mode_reference_rule(oracle_lib):
    """Reference stopping rule: emit boxes with width(x_1) < tol at the last cycle."""
    p = P.instance(P.COSQUAD, 4, 99, tol=0.0, split=(4, 2))
    p.stop_mode = P.STOP_WIDTH
    p.width_tol = 1e-3
    p.ub_init = 1e6
    r = oracle_lib.solve(p, box_cap=4096, trace_cap=4096)
    assert r.status == 0 and r.n_boxes >= 1
    assert r.lb <= 0.0 <= r.ub
    w = r.boxes[:, 1] - r.boxes[:, 0]
    assert np.all(w < 1e-3)
    assert r.pool_size == 0
