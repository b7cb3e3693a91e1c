"""CPU: the admission and scheduling logic of ``ServingEngine.run`` with the device pools replaced by
fakes (a pool's chunk completes as soon as it is launched): requests are placed first come, first
served into slots of the pool of their key, a new pool is created only when the planned bytes of
the pools in flight stay within the budget, empty pools give their bytes back when the budget is
needed, a pool that alone exceeds the budget is refused, members leave at their last step and a
diverged member leaves with that status. Also the pool keys of the request stream."""
from __future__ import annotations

import types

import pytest

from conatus_gb300 import serving


class _FakePool:
    created: list = []

    def __init__(self, key, slots, precision="fp64", chunk=500, unroll=25):
        self.key, self.slots = key, slots
        self.footprint = key[1]
        self.members, self.pending = [], []
        self.chunk = chunk
        _FakePool.created.append(key)

    def free(self):
        return self.slots - len(self.members) - len(self.pending)

    def empty(self):
        return not self.members and not self.pending

    def place(self, req):
        self.pending.append(req)

    def idle(self):
        return True

    def boundary(self, now):
        left = []
        for m in list(self.members):
            if m.remaining == 0 or m.params.get("diverge_at") == m.steps - m.remaining:
                m.status = "done" if m.remaining == 0 else "nonfinite"
                m.finished = now()
                m.result = m.rid
                left.append(m)
                self.members.remove(m)
        for r in self.pending:
            r.remaining = r.steps
            r.status = "running"
            self.members.append(r)
        self.pending = []
        return left

    def launch(self):
        if not self.members:
            return 0
        n = min(min(m.remaining for m in self.members), self.chunk, serving.CHECK_EVERY)
        for m in self.members:
            m.remaining -= n
        return n


def _fake_torch():
    return types.SimpleNamespace(cuda=types.SimpleNamespace(synchronize=lambda: None))


@pytest.fixture
def fake_pools(monkeypatch):
    _FakePool.created = []
    monkeypatch.setattr(serving, "Pool", _FakePool)
    monkeypatch.setattr(serving, "_torch", _fake_torch)
    # key = (kind, planned bytes of its pool, tag); a pool's bytes are its key's second entry
    monkeypatch.setattr(serving, "pool_key", lambda r: ("burgers", r.params["bytes"], r.params.get("tag", 0)))
    monkeypatch.setattr(serving, "plan_pool", lambda key, slots, precision="fp64": key[1])
    return _FakePool


def _requests(specs, steps=1200):
    return [serving.Request(i, "burgers", dict(sp), steps, 0.001 * i) for i, sp in enumerate(specs)]


def test_members_share_pools_first_come_first_served(fake_pools):
    reqs = _requests([{"bytes": 40}] * 5 + [{"bytes": 30, "tag": 1}] * 3)
    eng = serving.ServingEngine(budget_bytes=100, slots={"burgers": 4}, keep_results=True)
    out = eng.run(reqs, realtime=False)
    assert out["requests"] == 8 and out["steps"] == 8 * 1200 and out["nonfinite"] == 0
    # 5 requests of one key in pools of 4 slots: two pools (80 bytes); the other key's pool (30
    # bytes) waits for them to empty, and so do the requests behind it
    assert sorted(fake_pools.created) == [("burgers", 30, 1), ("burgers", 40, 0), ("burgers", 40, 0)]
    assert out["peak_planned_bytes"] == 80 and out["peak_members"] == 5 and out["budget_waits"] > 0
    adm = [r.admitted for r in sorted(reqs, key=lambda r: r.rid)]
    assert adm == sorted(adm)
    assert [r.result for r in reqs] == list(range(8))


def test_budget_bounds_the_pools_in_flight(fake_pools):
    """Six requests of six keys of 50 bytes each under a 100-byte budget: two pools at a time; a
    pool left empty is released when the next one needs its bytes."""
    reqs = _requests([{"bytes": 50, "tag": k} for k in range(6)], steps=300)
    eng = serving.ServingEngine(budget_bytes=100, slots={"burgers": 4})
    out = eng.run(reqs, realtime=False)
    assert out["requests"] == 6 and out["peak_planned_bytes"] == 100
    assert out["budget_waits"] > 0 and len(fake_pools.created) == 6


def test_pool_above_budget_refused(fake_pools):
    eng = serving.ServingEngine(budget_bytes=100)
    with pytest.raises(MemoryError):
        eng.run(_requests([{"bytes": 50}, {"bytes": 150, "tag": 1}]), realtime=False)


def test_diverged_member_leaves_with_its_status(fake_pools):
    reqs = _requests([{"bytes": 10}, {"bytes": 10, "diverge_at": 200}, {"bytes": 10}], steps=500)
    eng = serving.ServingEngine(budget_bytes=100, slots={"burgers": 8})
    out = eng.run(reqs, realtime=False)
    assert out["requests"] == 3 and out["nonfinite"] == 1 and out["steps"] == 1000
    assert [r.status for r in reqs] == ["done", "nonfinite", "done"]


def test_chunks_end_on_checks_and_last_steps(fake_pools):
    """Members advance in chunks that end at every member's last step and at least every 100 steps
    (the finite-state check's cadence)."""
    seen = []
    orig = _FakePool.launch

    def launch(self):
        n = orig(self)
        seen.append(n)
        return n

    _FakePool.launch = launch
    try:
        reqs = _requests([{"bytes": 10}] * 2, steps=250)
        reqs[1].steps = 130
        serving.ServingEngine(budget_bytes=100, slots={"burgers": 4}).run(reqs, realtime=False)
    finally:
        _FakePool.launch = orig
    assert max(seen) <= serving.CHECK_EVERY and 30 in seen


def test_pool_keys_of_the_stream():
    """Requests of one template, resolution and time step share a key; RB steps sit on the 1e-4 / 4^k
    ladder below the advective limit."""
    import math
    reqs = serving.poisson_stream(400, seed=3)
    for r in reqs:
        k = serving.pool_key(r)
        dt = k[-1]
        if r.kind == "rb":
            limit = 0.25 * (serving.RB_LX / r.params["Nx"]) / math.sqrt(r.params["Ra"])
            assert dt <= limit * (1 + 1e-12) and (limit < 4 * dt or (dt == 1e-4 and limit >= 1e-4))
            assert k[:3] == ("rb", r.params["Nz"], r.params["Nx"])
        else:
            assert k == (r.kind, r.params["N"], serving.DT[r.kind])
    assert len({serving.pool_key(r) for r in reqs}) < len(reqs) / 4
