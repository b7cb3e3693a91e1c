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
    monkeypatch.setattr(autotune, "partitioned_schedules", lambda: set())
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


def test_partitioned_schedule_only_when_opted_into(fake, monkeypatch):
    """The partitioned solve (here the fastest, schedule 1) is timed only for a DeviceProblem that
    opts into it; the two choices are cached apart."""
    monkeypatch.setattr(autotune, "partitioned_schedules", lambda: {1})
    fs = [_Handle(127, 262)]
    times = autotune.tune_solve(_Dev(fake), (1.0, 0.5), fs)
    assert 1 not in times and fs[0].schedule == 2
    dev = _Dev(fake)
    dev.partitioned = True
    fs2 = [_Handle(127, 262)]
    times = autotune.tune_solve(dev, (1.0, 0.5), fs2)
    assert 1 in times and fs2[0].schedule == 1
    assert len(autotune.cache()) == 2


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
    """The FP32 form's two refinement groups (two streams): (bucket, first system, end system)
    parts of about equal work (systems x length), every system in exactly one group; a bucket that
    outweighs all the others is split at a warp-group boundary, a shared pair's partner follows its
    primary."""
    from conatus_gb300.ivp import DeviceProblem
    B = types.SimpleNamespace

    def stub(nsys, ns, shared):
        st = B(nsys=nsys, tpl=B(buckets=[B(n=n) for n in ns]), _groups=None, shared=shared)
        st._with_partners = lambda parts: DeviceProblem._with_partners(st, parts)
        return st

    def covered(st, g):
        seen = {}
        for part in sum((st._with_partners(grp) for grp in g), []):
            bi, s0, s1 = part
            seen.setdefault(bi, []).append((s0, s1))
        for bi, ns in enumerate(st.nsys):
            r = sorted(seen[bi])
            assert r[0][0] == 0 and r[-1][1] == ns and all(a[1] == b[0] for a, b in zip(r, r[1:])), (bi, r)

    def work(st, grp):
        return sum((s1 - s0) * st.tpl.buckets[bi].n for bi, s0, s1 in st._with_partners(grp))

    st = stub([1, 95, 95, 9025, 9025], [523, 522, 522, 522, 522], {})
    g = DeviceProblem._refine_groups(st)
    covered(st, g)
    assert len(g) == 2 and abs(work(st, g[0]) - work(st, g[1])) <= 96 * 522
    one = stub([127], [262], {})
    g = DeviceProblem._refine_groups(one)
    covered(one, g)
    assert len(g) == 2 and abs(work(one, g[0]) - work(one, g[1])) <= 2 * 262     # split at an even system
    assert all(s0 % 2 == 0 for grp in g for _, s0, _ in grp)
    # a shared pair (bucket 4 solved with bucket 3's factors): bucket 3 split between the groups,
    # its partner's residual over the same systems
    pair = stub([1, 95, 95, 9025, 9025], [523, 522, 522, 522, 522], {4: 3})
    g = DeviceProblem._refine_groups(pair)
    covered(pair, g)
    assert all(bi != 4 for grp in g for bi, _, _ in grp)
    assert abs(work(pair, g[0]) - work(pair, g[1])) <= 2 * 522
