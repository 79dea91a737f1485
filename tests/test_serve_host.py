"""Host logic of the serving loop against a fake engine (no GPU): arrival
ordering, admission only while slots are free, collection, latency accounting."""
from types import SimpleNamespace

import pytest

from gpugo_gb300 import problems as P
from gpugo_gb300.serve import serve


class FakeEngine:
    """A solve needs `iters` runs of one slice; at most `slots` are resident."""

    def __init__(self, slots, iters):
        self.slots, self.iters = slots, iters
        self.resident = {}
        self.next = 1
        self.runs = 0
        self.max_resident = 0
        self.admit_order = []

    def submit(self, p, box_cap=4):
        if len(self.resident) >= self.slots:
            return None
        t = self.next
        self.next += 1
        self.resident[t] = [self.iters, p]
        self.admit_order.append(p.tag)
        self.max_resident = max(self.max_resident, len(self.resident))
        return t

    def submit_many(self, probs, box_cap=4):
        """gpugo_submit_batch's contract: the admitted prefix's tickets."""
        out = []
        for p in probs:
            t = self.submit(p, box_cap)
            if t is None:
                break
            out.append(t)
        return out

    def run(self, k):
        self.runs += 1
        for v in self.resident.values():
            v[0] -= 1
        return sum(v[0] > 0 for v in self.resident.values())

    def poll(self):
        out = []
        for t in [t for t, v in self.resident.items() if v[0] <= 0]:
            p = self.resident.pop(t)[1]
            out.append((t, SimpleNamespace(boxes_bounded=10, certified=True, tag=p.tag)))
        return out

    def stats(self):
        return {"total_run_ms": float(self.runs), "kernel_launches": self.runs, "iterations": self.runs}

    def close(self):
        pass


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 0.001
        return self.t


def test_admission_respects_slots_and_arrival_order():
    stream = [(0.0005 * i, P.instance(P.COSQUAD, 2, i, tag=f"q{i}")) for i in range(20)]
    eng = FakeEngine(slots=3, iters=2)
    rep = serve(stream, engine=eng, clock=FakeClock())
    assert eng.max_resident == 3
    assert eng.admit_order == [f"q{i}" for i in range(20)]
    assert rep.certified == 20 and rep.boxes == 200
    for r in rep.records:
        assert r.admitted >= r.arrival and r.finished > r.admitted
        assert r.result.tag == f"q{r.index}"
    assert rep.p99_ms >= rep.p50_ms > 0


def test_solve_all_admits_by_shape_and_returns_input_order():
    """Engine.solve_all (host logic, run on a fake engine): admission ordered by
    (family, n), refills as slots free up, results in the caller's order."""
    import gpugo_gb300 as G
    probs = P.config4(count=40, seed=5, nmax=30)
    for i, p in enumerate(probs):
        p.tag = f"p{i}"
    fake = FakeEngine(slots=7, iters=3)
    res = G.Engine.solve_all(fake, probs, iters_per_run=1)
    assert [r.tag for r in res] == [p.tag for p in probs]
    shapes = [(p.family, p.n) for p in sorted(probs, key=lambda q: (q.family, q.n))]
    by_tag = {p.tag: (p.family, p.n) for p in probs}
    assert [by_tag[t] for t in fake.admit_order] == shapes
    assert fake.max_resident == 7
    fake2 = FakeEngine(slots=7, iters=3)
    G.Engine.solve_all(fake2, probs, iters_per_run=1, group_by_shape=False)
    assert fake2.admit_order == [p.tag for p in probs]


class PickyEngine(FakeEngine):
    """Refuses problems tagged "bad" like the library refuses an invalid
    description, and never has room for problems tagged "huge"."""

    def submit(self, p, box_cap=4):
        import gpugo_gb300 as G
        if p.tag.startswith("bad"):
            raise G.GpugoError(-1, "gpugo_submit")
        if p.tag.startswith("huge"):
            return None
        return super().submit(p, box_cap)


def test_refused_requests_are_answered_and_the_stream_goes_on():
    """Host-side fault injection: an invalid request and one that cannot fit an
    empty engine are answered with their error; every other request is served
    in arrival order and the latency figures cover the served ones only."""
    tags = ["q0", "bad1", "q2", "q3", "huge4", "q5", "bad6", "q7"]
    stream = [(0.0005 * i, P.instance(P.COSQUAD, 2, i, tag=t)) for i, t in enumerate(tags)]
    eng = PickyEngine(slots=2, iters=2)
    rep = serve(stream, engine=eng, clock=FakeClock())
    served = [r for r in rep.records if r.result is not None]
    assert [r.result.tag for r in served] == ["q0", "q2", "q3", "q5", "q7"]
    assert eng.admit_order == ["q0", "q2", "q3", "q5", "q7"]
    refused = {r.index: r.error for r in rep.records if r.result is None}
    assert set(refused) == {1, 4, 6}
    assert "invalid" in refused[1] and "empty engine" in refused[4]
    assert rep.rejected == 3 and rep.certified == 5 and rep.summary()["rejected"] == 3
    assert rep.p99_ms >= rep.p50_ms > 0


def test_device_failure_in_admission_is_not_swallowed():
    import pytest
    import gpugo_gb300 as G

    class Broken(FakeEngine):
        def submit(self, p, box_cap=4):
            raise G.GpugoError(-2, "gpugo_submit")

    stream = [(0.0, P.instance(P.COSQUAD, 2, 1, tag="q0"))]
    with pytest.raises(G.GpugoError):
        serve(stream, engine=Broken(slots=2, iters=1), clock=FakeClock())


def test_shape_order_groups_waiting_requests():
    """order="shape": requests waiting together take the free slots grouped by
    (family, n), then by arrival; every request is still served once."""
    fams = [P.CHAINED, P.COSQUAD, P.CHAINED, P.COSQUAD, P.EXPSQRT, P.COSQUAD]
    ns = [5, 3, 4, 3, 2, 2]
    stream = [(0.0, P.instance(f, n, i, tag=f"q{i}")) for i, (f, n) in enumerate(zip(fams, ns))]
    eng = FakeEngine(slots=2, iters=1)
    rep = serve(stream, max_slots=2, slice_iters=1, engine=eng, clock=FakeClock(), order="shape")
    assert sorted(eng.admit_order) == sorted(f"q{i}" for i in range(6))
    assert eng.admit_order[:2] == ["q5", "q1"]          # cosquad n=2, then cosquad n=3 (earlier arrival)
    assert rep.certified == 6
    with pytest.raises(ValueError):
        serve(stream, engine=FakeEngine(2, 1), order="random")
