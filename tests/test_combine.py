"""Result-box merging (rosenbrock50.py:926-1049): oracle against the reference's
own combine / connectivity (golden vectors), GPU against the oracle."""
import numpy as np
import pytest

import gpugo_gb300 as G


def _cases(golden):
    n = golden["combine_n"]
    tol = golden["combine_tol"]
    bo, ro = golden["combine_box_offsets"], golden["combine_root_offsets"]
    boxes, roots = golden["combine_boxes"], golden["combine_roots"]
    pb = pr = 0
    for c in range(len(n)):
        k, m, nn = bo[c + 1] - bo[c], ro[c + 1] - ro[c], int(n[c])
        yield (nn, float(tol[c]), boxes[pb:pb + 2 * nn * k].reshape(k, nn, 2),
               roots[pr:pr + 2 * nn * m].reshape(m, nn, 2))
        pb += 2 * nn * k
        pr += 2 * nn * m


def test_oracle_combine_matches_reference(golden, oracle_lib):
    merged = 0
    for n, tol, boxes, roots in _cases(golden):
        got = oracle_lib.combine(boxes, tol)
        assert got.shape == roots.shape
        assert np.array_equal(got, roots)     # values; -0 and +0 compare equal
        merged += boxes.shape[0] - roots.shape[0]
    assert merged > 50                         # the vectors exercise merging


def test_oracle_combine_edge_cases(oracle_lib):
    assert oracle_lib.combine(np.zeros((0, 3, 2)), 1e-3).shape == (0, 3, 2)
    one = np.array([[[0.0, 1e-5], [2.0, 2.00001]]])
    assert np.array_equal(oracle_lib.combine(one, 1e-3), one)
    # a box wider than the tolerance joins only a root that contains it
    wide = np.array([[[0.0, 0.1]], [[0.05, 0.2]], [[0.01, 0.02]]])
    r = oracle_lib.combine(wide, 1e-3)
    assert r.shape[0] == 2 and np.array_equal(r[0], wide[0])


@pytest.mark.gpu
def test_gpu_combine_matches_oracle(golden, oracle_lib):
    for n, tol, boxes, roots in _cases(golden):
        assert np.array_equal(G.combine(boxes, tol), roots)
    rng = np.random.default_rng(3)
    for n in (1, 4, 40):
        lo = rng.uniform(-1, 1, size=(3000, n)) * 2e-3 + rng.integers(0, 4, size=(3000, 1))
        w = rng.uniform(0, 5e-4, size=(3000, n))
        boxes = np.stack([lo, lo + w], axis=2)
        assert np.array_equal(G.combine(boxes, 1e-3), oracle_lib.combine(boxes, 1e-3))
    assert G.combine(np.zeros((0, 2, 2)), 1e-3).shape == (0, 2, 2)
