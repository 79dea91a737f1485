"""Autotuner search logic on the CPU (a fake timer), and one tuning run on the GPU."""
import pytest

import gpugo_gb300 as G
from gpugo_gb300 import autotune as A
from gpugo_gb300 import problems as P


def _fake_timer(calls):
    def timer(problems, cfg):
        calls.append((len(problems), cfg, tuple(sorted({(p.wid, p.group) for p in problems}))))
        t = 1.0 + 0.1 * A.ENGINE_CONFIGS.index(cfg)          # the first config is fastest
        if cfg == A.ENGINE_CONFIGS[3]:
            t = 0.5                                          # ... unless lane mode
        t += sum(abs(p.wid - 5) + abs(p.group - 5) for p in problems) * 1e-3   # prefers (5, 5)
        return t
    return timer


def test_tune_picks_fastest_engine_then_fanout():
    probs = P.config4(count=96, seed=5, nmax=64)
    calls = []
    r = A.tune(probs, sample=32, timer=_fake_timer(calls), per_class=8)
    assert r.engine == A.ENGINE_CONFIGS[3]
    engine_trials = [t for t in r.trials if t["kind"] == "engine"]
    assert len(engine_trials) == len(A.ENGINE_CONFIGS)
    assert all(t["instances"] == 32 for t in engine_trials)
    # every fan-out trial ran with the winning engine configuration
    assert all(c[1] == A.ENGINE_CONFIGS[3] for c in calls[len(A.ENGINE_CONFIGS):])
    for cls, split in r.fanout.items():
        assert split == (5, 5), cls
    # apply changes only instances inside a tuned class
    tuned = r.apply(probs)
    for p, q in zip(probs, tuned):
        if r.split_for(p.n) is None:
            assert (q.wid, q.group) == (p.wid, p.group)
        else:
            assert (q.wid, q.group) == (5, 5) and q.n == p.n and (q.coef == p.coef).all()
    assert "engine" in r.to_json()


def test_sample_keeps_order_and_size():
    probs = P.config4(count=50, seed=6, nmax=16)
    s = A.sample_problems(probs, 10)
    assert len(s) == 10 and s[0] is probs[0]
    assert A.sample_problems(probs, 80) == probs


@pytest.mark.gpu
def test_tune_on_gpu_small():
    probs = P.config4(count=48, seed=7, nmax=24)
    r = A.tune(probs, sample=16, per_class=4, configs=A.ENGINE_CONFIGS[:2],
               fanout_options=((3, 6), (3, 8)), n_classes=((8, 24),))
    assert r.engine in A.ENGINE_CONFIGS[:2]
    assert all(t["seconds"] > 0 for t in r.trials)
    tuned = r.apply(probs)
    with G.Engine(max_slots=len(tuned), arena_bytes=4 << 30, threads=r.engine.threads,
                  blocks_per_sm=r.engine.blocks_per_sm, cand_mode=r.engine.cand_mode) as eng:
        res = eng.solve_all(tuned, box_cap=2)
    assert all(x.certified for x in res)
    for p, x in zip(tuned, res):
        assert x.lb <= 0.0 <= x.ub + 1e-12 and x.ub - x.lb <= p.gap_tol
