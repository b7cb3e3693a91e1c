"""CPU: the admission and retirement logic of ``ServingEngine.run`` with the device runs replaced by
fakes (a run's chunk completes as soon as it is launched): requests are admitted first come, first
served, the planned bytes of the runs in flight never exceed the budget, finished runs give their
bytes back, and a request that alone exceeds the budget is refused."""
from __future__ import annotations

import types

import pytest

from conatus_gb300 import serving


class _FakeSession:
    log: list = []

    def __init__(self, prep, precision="fp64"):
        self.req = prep.req
        self.footprint = prep.bytes
        self.remaining = prep.req.steps
        _FakeSession.log.append(prep.req.rid)

    def launch(self, chunk, unroll):
        self.remaining -= min(chunk, self.remaining)

    def idle(self):
        return True

    def finite(self):
        return True

    def result(self):
        return self.req.rid


def _fake_torch():
    cuda = types.SimpleNamespace(synchronize=lambda: None)
    return types.SimpleNamespace(cuda=cuda)


@pytest.fixture
def fake_device(monkeypatch):
    _FakeSession.log = []
    monkeypatch.setattr(serving, "Session", _FakeSession)
    monkeypatch.setattr(serving, "_torch", _fake_torch)
    monkeypatch.setattr(serving, "prepare",
                        lambda req, precision="fp64": serving.Prepared(req, None, None, req.params["bytes"]))
    return _FakeSession


def _requests(sizes, steps=1200, kind="burgers"):
    return [serving.Request(i, kind, {"bytes": b}, steps, 0.001 * i) for i, b in enumerate(sizes)]


def test_first_come_first_served_within_budget(fake_device):
    sizes = [40, 30, 50, 20, 60, 10, 45, 35]
    eng = serving.ServingEngine(budget_bytes=100, chunk=500, unroll=50, free_batch=1)
    out = eng.run(_requests(sizes), realtime=False)
    assert out["requests"] == len(sizes) and out["steps"] == 1200 * len(sizes)
    assert fake_device.log == list(range(len(sizes)))            # admission in arrival order
    assert out["peak_planned_bytes"] <= 100
    assert out["peak_active"] >= 2                                # runs do overlap
    assert out["nonfinite"] == 0 and out["by_kind"]["burgers"] == len(sizes)


def test_budget_bounds_the_runs_in_flight(fake_device):
    eng = serving.ServingEngine(budget_bytes=100, chunk=100, unroll=50, free_batch=1)
    out = eng.run(_requests([50] * 6), realtime=False)
    assert out["requests"] == 6
    assert out["peak_active"] == 2 and out["peak_planned_bytes"] == 100


def test_max_active_bounds_the_runs_in_flight(fake_device):
    eng = serving.ServingEngine(budget_bytes=1e9, chunk=100, unroll=50, max_active=3)
    out = eng.run(_requests([1] * 10), realtime=False)
    assert out["requests"] == 10 and out["peak_active"] == 3


def test_batched_release_frees_before_refusing(fake_device):
    """With retirement batched (free_batch large), a request that does not fit still gets in once
    the finished runs are released."""
    eng = serving.ServingEngine(budget_bytes=100, chunk=2000, unroll=50, free_batch=1000)
    out = eng.run(_requests([60, 60, 60]), realtime=False)
    assert out["requests"] == 3 and out["peak_planned_bytes"] <= 100


def test_request_above_budget_refused(fake_device):
    eng = serving.ServingEngine(budget_bytes=100)
    with pytest.raises(MemoryError):
        eng.run(_requests([50, 150]), realtime=False)


def test_results_kept_on_request(fake_device):
    eng = serving.ServingEngine(budget_bytes=100, keep_results=True)
    reqs = _requests([10, 20, 30])
    eng.run(reqs, realtime=False)
    assert [r.result for r in reqs] == [0, 1, 2]
    assert all(r.finished >= r.admitted >= r.arrival for r in reqs)
