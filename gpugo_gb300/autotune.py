"""Autotuner for the batched engine: block size, candidates per warp and split fan-out.

The engine's throughput on a batch depends on three choices that no formula
settles on this part (an FP64 warp instruction costs the same for 1 or 32 active
lanes, and SMs share nothing but L2):

* **block size** -- 256 or 512 threads per block, one or two blocks per SM;
* **candidates per warp** -- a whole warp per candidate child (its sample passes
  side by side) or one lane per candidate (32 per warp), or the engine's
  automatic switch by queue length (``gpugo_engine_cfg.cand_mode``);
* **fan-out** -- the split rule ``(wid, group)`` of generated instances, i.e.
  ``wid**group`` children per iteration.  Any split gives a rigorous enclosure;
  it changes the number of iterations and boxes, not the guarantee.

:func:`tune` times each engine configuration on a sample of the workload (whole
solves, device time from the engine's CUDA events) and then, with the best one,
each fan-out option per dimension class; it returns the winners and every trial.
The timing function is a parameter so that the search logic is tested on the CPU.
"""
from __future__ import annotations

import dataclasses
import json
import math
from dataclasses import dataclass, field
from typing import Callable, Sequence

from . import _lib
from .problems import Problem

# split options tried for instances of n >= 8 (odd wid: see problems.default_split)
FANOUT_OPTIONS: tuple[tuple[int, int], ...] = ((3, 4), (3, 5), (3, 6), (3, 8), (5, 4), (5, 5), (3, 10))
# dimension classes for the fan-out choice (instances with n < 8 keep the default table)
N_CLASSES: tuple[tuple[int, int], ...] = ((8, 16), (17, 32), (33, 64), (65, 4096))
# the small dimensions, one class each, with their own options (the default
# table's split first; odd wid, wid^min(group, n) children per iteration)
SMALL_FANOUT: dict[tuple[int, int], tuple[tuple[int, int], ...]] = {
    (2, 2): ((31, 2), (15, 2), (9, 2), (7, 2), (5, 2)),
    (3, 3): ((9, 3), (7, 3), (5, 3), (3, 3)),
    (4, 4): ((7, 4), (5, 4), (3, 4)),
    (5, 5): ((5, 5), (3, 5), (5, 4), (3, 4)),
    (6, 6): ((5, 6), (3, 6), (5, 5), (3, 5), (5, 4)),
    (7, 7): ((3, 7), (3, 6), (5, 5), (3, 5)),
}


@dataclass(frozen=True)
class EngineConfig:
    threads: int = 256
    blocks_per_sm: int = 0        # 0: as many as fit (two of 256 threads)
    cand_mode: int = _lib.CAND_AUTO

    def label(self) -> str:
        mode = {_lib.CAND_AUTO: "auto", _lib.CAND_WARP: "warp", _lib.CAND_LANE: "lane"}[self.cand_mode]
        return f"t{self.threads}-b{self.blocks_per_sm or 'max'}-{mode}"


# The fan-out this tuner chose on a GB300 for the mixed batch of generated
# instances (families F1-F4, n log-uniform in 2..64 and 2..128): three parts per
# coordinate, 3^5 children per iteration for n <= 16 and 3^6 above; for the
# small dimensions the default table's split except at n = 5 and n = 6, where
# three parts per coordinate (3^5, 3^6 children) certified the class's sample
# 7x and 14x faster than five parts (5^5, 5^6).  Workloads that must solve
# identical problems in several runs (a GPU run and a CPU baseline) apply this
# table instead of tuning the fan-out again.
TUNED_FANOUT: dict[tuple[int, int], tuple[int, int]] = {
    (2, 2): (31, 2), (3, 3): (9, 3), (4, 4): (7, 4), (5, 5): (3, 5), (6, 6): (3, 6), (7, 7): (3, 7),
    (8, 16): (3, 5), (17, 32): (3, 6), (33, 64): (3, 6), (65, 4096): (3, 6)}

ENGINE_CONFIGS: tuple[EngineConfig, ...] = (
    EngineConfig(256, 0, _lib.CAND_AUTO),
    EngineConfig(256, 1, _lib.CAND_AUTO),
    EngineConfig(512, 0, _lib.CAND_AUTO),
    EngineConfig(256, 0, _lib.CAND_LANE),
    EngineConfig(256, 0, _lib.CAND_WARP),
)


@dataclass
class TuneResult:
    engine: EngineConfig
    fanout: dict[tuple[int, int], tuple[int, int]]      # n class -> (wid, group)
    trials: list[dict] = field(default_factory=list)

    def split_for(self, n: int) -> tuple[int, int] | None:
        for (lo, hi), split in self.fanout.items():
            if lo <= n <= hi:
                return split
        return None

    def apply(self, problems: Sequence[Problem]) -> list[Problem]:
        """Copies of ``problems`` (instances whose split is free to choose) with the
        tuned fan-out; instances outside the tuned classes are returned unchanged."""
        out = []
        for p in problems:
            split = self.split_for(p.n)
            out.append(p if split is None else dataclasses.replace(p, wid=split[0], group=split[1]))
        return out

    def to_json(self) -> str:
        return json.dumps({"engine": dataclasses.asdict(self.engine),
                           "fanout": {f"{lo}-{hi}": list(v) for (lo, hi), v in self.fanout.items()},
                           "trials": self.trials})


def apply_fanout(problems: Sequence[Problem], fanout: dict[tuple[int, int], tuple[int, int]] = None) -> list[Problem]:
    """``problems`` with a fixed fan-out table applied (by default the tuned one)."""
    return TuneResult(EngineConfig(), dict(TUNED_FANOUT if fanout is None else fanout)).apply(problems)


def time_engine(problems: Sequence[Problem], cfg: EngineConfig, arena_bytes: int = 16 << 30) -> float:
    """Device seconds to certify ``problems`` in one engine (all admitted at once
    when they fit, refilled otherwise)."""
    from . import Engine
    with Engine(max_slots=max(1, len(problems)), arena_bytes=arena_bytes, threads=cfg.threads,
                blocks_per_sm=cfg.blocks_per_sm, cand_mode=cfg.cand_mode) as eng:
        eng.solve_all(list(problems[:1]), box_cap=1)        # first launch outside the measurement
        st0 = eng.stats()
        eng.solve_all(list(problems), box_cap=1)
        st1 = eng.stats()
    return (st1["total_run_ms"] - st0["total_run_ms"]) * 1e-3


def sample_problems(problems: Sequence[Problem], k: int) -> list[Problem]:
    """Every (len/k)-th problem: a deterministic sample that keeps the mix."""
    if k >= len(problems):
        return list(problems)
    step = len(problems) / k
    return [problems[int(i * step)] for i in range(k)]


def tune(problems: Sequence[Problem], sample: int = 512, configs: Sequence[EngineConfig] = ENGINE_CONFIGS,
         fanout_options: Sequence[tuple[int, int]] | dict = FANOUT_OPTIONS,
         n_classes: Sequence[tuple[int, int]] = N_CLASSES, per_class: int = 16,
         timer: Callable[[Sequence[Problem], EngineConfig], float] = time_engine) -> TuneResult:
    """Pick the engine configuration, then the fan-out per dimension class.
    ``fanout_options`` is one list of splits for every class, or a dict of
    class -> splits (a class missing from it takes FANOUT_OPTIONS)."""
    trials: list[dict] = []
    base = sample_problems(problems, sample)
    best_cfg, best_t = configs[0], math.inf
    for cfg in configs:
        t = timer(base, cfg)
        trials.append({"kind": "engine", "config": cfg.label(), "instances": len(base), "seconds": t})
        if t < best_t:
            best_cfg, best_t = cfg, t
    fanout: dict[tuple[int, int], tuple[int, int]] = {}
    for lo, hi in n_classes:
        members = [p for p in problems if lo <= p.n <= hi]
        if not members:
            continue
        members = sample_problems(members, per_class)
        best_split, best_ts = None, math.inf
        options = fanout_options.get((lo, hi), FANOUT_OPTIONS) if isinstance(fanout_options, dict) else fanout_options
        for wid, group in options:
            if wid ** min(group, lo) > 2 ** 32:
                continue
            trial = [dataclasses.replace(p, wid=wid, group=group) for p in members]
            t = timer(trial, best_cfg)
            trials.append({"kind": "fanout", "n_class": [lo, hi], "split": [wid, group],
                           "instances": len(trial), "seconds": t})
            if t < best_ts:
                best_split, best_ts = (wid, group), t
        if best_split is not None:
            fanout[(lo, hi)] = best_split
    return TuneResult(best_cfg, fanout, trials)
