"""CPU: the selection logic of the solve-schedule autotuner with the device replaced by fakes (a
solve of schedule s takes a scripted time): the fastest candidate is kept for every handle of the
factor set, candidates that do not fit are skipped, results are cached per bucket shapes and
precision, and the environment override fixes the schedule without timing."""
from __future__ import annotations

import types

import pytest

from conatus_gb300 import autotune

COST = {-1: 9.0, 0: 4.0, 1: 2.5, 2: 3.0, 3: 7.0}


class _Clock:
    def __init__(self):
        self.t = 0.0


def _fake_torch(clock):
    class Event:
        def __init__(self, enable_timing=False):
            self.t = None

        def record(self, stream=None):
            self.t = clock.t

        def synchronize(self):
            pass

        def elapsed_time(self, other):
            return other.t - self.t

    class _Ctx:
        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

    cuda = types.SimpleNamespace(Event=Event, current_stream=lambda: "s0", stream=lambda s: _Ctx(),
                                 ExternalStream=lambda p: f"ext{p}")
    return types.SimpleNamespace(cuda=cuda)


class _Handle:
    def __init__(self, batch, n):
        self.batch, self.n, self.rank, self.kl, self.ku = batch, n, 6, 9, 22
        self.schedule = None


class _Dev:
    def __init__(self, clock, precision="fp64", refuse=()):
        self.clock, self.precision, self.refuse = clock, precision, set(refuse)
        self.solves = 0

    def zeros(self):
        return types.SimpleNamespace(fill_=lambda v: None)

    def _solve_with(self, fs, a, b, rhs, out, st):
        s = fs[0].schedule
        if s in self.refuse:
            raise ValueError("compact solve: system too large for shared memory")
        self.solves += 1
        self.clock.t += COST[s]


@pytest.fixture
def fake(monkeypatch):
    clock = _Clock()
    import conatus_gb300.ivp as ivp
    monkeypatch.setattr(ivp, "_torch", lambda: _fake_torch(clock))

    def apply(fs, sched):
        for h in fs:
            h.schedule = int(sched)
    monkeypatch.setattr(autotune, "apply", apply)
    monkeypatch.setattr(autotune, "schedules", lambda: sorted(COST))
    monkeypatch.setattr(autotune, "_CACHE", {})
    monkeypatch.delenv("CONATUS_GB300_SOLVE_SCHEDULE", raising=False)
    return clock


def test_fastest_kept_for_every_handle(fake):
    fs = [_Handle(9025, 522), _Handle(95, 522)]
    dev = _Dev(fake)
    times = autotune.tune_solve(dev, (1.0, 0.5), fs, reps=3)
    assert times == pytest.approx(COST)
    assert all(h.schedule == 1 for h in fs)
    assert dev.solves == len(COST) * 4                   # one warm-up and three timed per candidate


def test_candidates_that_do_not_fit_are_skipped(fake):
    fs = [_Handle(100, 74)]
    times = autotune.tune_solve(_Dev(fake, refuse={1, 2}), (1.0, 0.5), fs)
    assert set(times) == {-1, 0, 3} and fs[0].schedule == 0


def test_no_fitting_candidate_is_an_error(fake):
    with pytest.raises(ValueError, match="no solve schedule"):
        autotune.tune_solve(_Dev(fake, refuse=set(COST)), (1.0, 0.5), [_Handle(10, 74)])


def test_cached_per_shapes_and_precision(fake):
    fs = [_Handle(127, 262)]
    dev = _Dev(fake)
    autotune.tune_solve(dev, (1.0, 0.5), fs)
    n = dev.solves
    fs2 = [_Handle(127, 262)]
    autotune.tune_solve(dev, (2.0, 0.25), fs2)            # same shapes: from the cache
    assert dev.solves == n and fs2[0].schedule == 1
    autotune.tune_solve(_Dev(fake, precision="fp32"), (1.0, 0.5), [_Handle(127, 262)])
    autotune.tune_solve(dev, (1.0, 0.5), [_Handle(128, 262)])
    assert len(autotune.cache()) == 3


def test_environment_fixes_the_schedule(fake, monkeypatch):
    monkeypatch.setenv("CONATUS_GB300_SOLVE_SCHEDULE", "3")
    fs = [_Handle(10, 74)]
    dev = _Dev(fake)
    assert autotune.tune_solve(dev, (1.0, 0.5), fs) == {3: None}
    assert fs[0].schedule == 3 and dev.solves == 0


def test_refine_groups_balance_the_work():
    """The FP32 form's two refinement groups (two streams): buckets split largest first into two
    groups of about equal work (systems x length); every bucket in exactly one group."""
    from conatus_gb300.ivp import DeviceProblem
    B = types.SimpleNamespace
    stub = B(nsys=[1, 95, 95, 9025, 9025], tpl=B(buckets=[B(n=523)] + [B(n=522)] * 4), _groups=None,
             shared={})
    g = DeviceProblem._refine_groups(stub)
    assert sorted(sum(g, [])) == [0, 1, 2, 3, 4]
    w = [sum(stub.nsys[b] * stub.tpl.buckets[b].n for b in grp) for grp in g]
    assert len(g) == 2 and abs(w[0] - w[1]) <= 96 * 522
    one = B(nsys=[127], tpl=B(buckets=[B(n=262)]), _groups=None, shared={})
    assert DeviceProblem._refine_groups(one) == [[0]]
    # a shared pair (bucket 4 solved with bucket 3's factors) stays in one group
    pair = B(nsys=[1, 95, 95, 9025, 9025], tpl=B(buckets=[B(n=523)] + [B(n=522)] * 4), _groups=None,
             shared={4: 3})
    g = DeviceProblem._refine_groups(pair)
    assert sorted(sum(g, [])) == [0, 1, 2, 3, 4]
    assert any(3 in grp and 4 in grp for grp in g)
