"""Continuous batching on the GPU: requests arriving while others run are
admitted as slots free up, and each result is identical to solving the problem
alone (same enclosure bits, iterations, list size and boxes)."""
import numpy as np
import pytest

import gpugo_gb300 as G
from gpugo_gb300 import problems as P
from gpugo_gb300.serve import serve

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("with_codelists,order", [(False, "arrival"), (True, "arrival"), (False, "shape")],
                         ids=["builtin", "mixed", "builtin-shape-order"])
def test_served_results_match_solo(with_codelists, order):
    probs = P.config4(count=18, seed=91, nmax=16) + [P.config1(), P.config2()]
    if with_codelists:
        from gpugo_gb300 import objectives as O
        # code-list requests arrive between built-in ones: launches switch builds
        probs = [q for pair in zip(probs[:7], [O.problem(n, 5) for n in sorted(O.REFERENCE)]) for q in pair]
        probs += [O.as_codelist(P.config2())]
    for p in probs:
        p.max_iter = 2000
    stream = [(0.0002 * i, p) for i, p in enumerate(probs)]
    solo = [G.solve(p, box_cap=4) for p in probs]
    with G.Engine(max_slots=5, arena_bytes=1 << 30) as eng:
        rep = serve(stream, engine=eng, slice_iters=3, box_cap=4, order=order)
    assert rep.launches > len(probs) // 5          # solves were interleaved across several runs
    for p, a, rec in zip(probs, solo, rep.records):
        b = rec.result
        assert (a.lb, a.ub, a.iterations, a.status, a.pool_size, a.n_boxes) == \
               (b.lb, b.ub, b.iterations, b.status, b.pool_size, b.n_boxes), p.tag
        assert np.array_equal(a.boxes, b.boxes)
        assert rec.admitted >= rec.arrival and rec.finished >= rec.admitted
    assert rep.certified == len(probs)
