"""Serving: a request loop that admits IVP runs of different kinds and resolutions as they arrive.

Each request asks for ``steps`` IMEX steps of one model (Burgers, Kuramoto-Sivashinsky or 2D
Rayleigh-Benard, each with its own resolution and parameter). The engine

* plans each request's device bytes before allocating anything (``conatus_gb300.memory``) and admits
  it once it has arrived and fits the HBM budget left by the runs in flight (a request that does not
  fit waits; requests behind it wait too, so admission is first come, first served);
* keeps every admitted run resident (state, history ring, factored operators: one factor set in the
  steady state) and advances it in chunks of graph-replayed steps on its own CUDA stream, so that
  the chunks of all runs in flight overlap on the device and new runs join while others run
  (continuous batching: a run's slot and memory are released when its last chunk completes);
* records arrival, admission and completion times: p50/p99 completion latency (completion minus
  arrival) and aggregate steps/s.

The reference serves nothing: it runs one ``Simulation`` per process (python/conatus/model/run.py).
Each run's arithmetic is that of ``conatus_gb300.ivp.IVPSolver`` (Burgers, RB) or
``conatus_gb300.ensemble.FourierEnsemble`` with one member (KS), so a run gives the same result
alone and in the mix: streams change the order of launches of different runs, not the arithmetic
of one run.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from . import memory
from . import workloads as W
from .ivp import IVPSolver, _torch
from .template import ProblemTemplate

__all__ = ["Request", "poisson_stream", "prepare", "Session", "ServingEngine"]

BURGERS_N = tuple(range(64, 513, 32))     # resolutions with a parameter-linear template
RB_NZ = (32, 48, 64, 80, 96)
SCHEME = "SBDF2"
DT = {"burgers": 1e-4, "ks": 1e-2, "rb": 1e-4}


RB_LX = 2 * math.pi / 3.117


def time_step(req) -> float:
    """dt of a request: 1e-4 for Burgers, 1e-2 for KS; for RB an advective limit, a quarter of the
    grid spacing Lx/Nx over the free-fall velocity (Ra Pr)^(1/2) (thermal-diffusion units, Pr = 1),
    at most 1e-4. The explicit advection of SBDF2 at dt = 1e-4 diverges from Ra ~ 1e5 up (the
    oracle's own runs blow up within a few thousand steps)."""
    if req.kind == "rb":
        u_ff = math.sqrt(req.params["Ra"])
        return min(DT["rb"], 0.25 * (RB_LX / req.params["Nx"]) / u_ff)
    return DT[req.kind]


@dataclass
class Request:
    rid: int
    kind: str                     # "burgers" | "ks" | "rb"
    params: dict
    steps: int
    arrival: float                # seconds after the start of the stream
    admitted: float | None = None
    finished: float | None = None
    footprint: int = 0
    result: object = None


def poisson_stream(count: int, rate: float = 200.0, seed: int = 0, steps=(1000, 20000),
                   mix=(0.5, 0.3, 0.2)) -> list:
    """Poisson arrivals at ``rate`` per second (seeded exponential gaps): 50% Burgers (N uniform in
    64..512, rounded to the nearest multiple of 32; nu log-uniform in [1e-3, 1e-1]), 30% KS (L uniform
    in [22, 100], N = next power of two >= 2L), 20% 2D RB (Nz uniform in 32..96, rounded to the
    nearest of 32, 48, .., 96; Nx = 4 Nz; Ra log-uniform in [1e4, 1e7]; Pr = 1); steps uniform in
    ``steps`` (inclusive)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate)
        u = rng.uniform()
        nsteps = int(rng.integers(steps[0], steps[1] + 1))
        if u < mix[0]:
            n = int(rng.integers(64, 513))
            n = min(BURGERS_N, key=lambda x: abs(x - n))
            out.append(Request(i, "burgers", dict(N=n, nu=float(10 ** rng.uniform(-3, -1))), nsteps, t))
        elif u < mix[0] + mix[1]:
            L = float(rng.uniform(22, 100))
            out.append(Request(i, "ks", dict(L=L, N=1 << int(math.ceil(math.log2(2 * L)))), nsteps, t))
        else:
            nz = int(rng.integers(32, 97))
            nz = min(RB_NZ, key=lambda x: abs(x - nz))
            out.append(Request(i, "rb", dict(Nz=nz, Nx=4 * nz, Ra=float(10 ** rng.uniform(4, 7))), nsteps, t))
    return out


_TEMPLATES: dict = {}


def _template(name: str) -> ProblemTemplate:
    t = _TEMPLATES.get(name)
    if t is None:
        t = _TEMPLATES[name] = W.load_template(name)
    return t


@dataclass
class Prepared:
    """Host-side set-up of a request: its problem, initial state and planned device bytes."""
    req: Request
    problem: object
    state: list
    bytes: int


def prepare(req: Request, precision: str = "fp64") -> Prepared:
    """Problem instance, seeded initial state and planned device bytes of a request (no device
    work)."""
    p = req.params
    if req.kind == "ks":
        return Prepared(req, None, None, memory.plan_fourier_ensemble([p["N"]], SCHEME)["total"])
    if req.kind == "burgers":
        P = _template(f"burgers_n{p['N']}_nu").instantiate(None, None, {"nu": p["nu"]})
        C0 = W.burgers_state(P)
    elif req.kind == "rb":
        P = _template(f"rb_nz{p['Nz']}_ra").instantiate([p["Nx"]], None, {"Ra": p["Ra"]})
        C0 = W.rayleigh_benard_state(P, req.rid)
    else:
        raise ValueError(req.kind)
    return Prepared(req, P, C0, memory.plan_ivp(P, SCHEME, precision, factor_sets=1)["total"])


class Session:
    """One admitted run, resident on the device."""

    def __init__(self, prep: Prepared, precision: str = "fp64"):
        torch = _torch()
        self.req = req = prep.req
        if req.kind == "ks":
            from .ensemble import FourierEnsemble
            p = req.params
            self.solver = FourierEnsemble(_template("ks"), [p["N"]], [p["L"]], scheme=SCHEME, dt=time_step(req),
                                          precision=precision)
            self.solver.set_state(self.solver.random_state(seed=req.rid))
        else:
            self.solver = IVPSolver(prep.problem, scheme=SCHEME, dt=time_step(req), precision=precision,
                                    factor_sets=1)
            self.solver.set_state(prep.state)
        # one wait for the initial state (copied on torch's stream), then the run's stream is on
        # its own: runs in flight do not wait on one another
        self.solver.stream.wait_stream(torch.cuda.current_stream())
        self.solver.join = False
        if hasattr(self.solver, "fork"):
            self.solver.fork = False            # runs in flight already fill the device
            self.solver.dev.overlap_refine = False
        self.footprint = prep.bytes
        self.remaining = req.steps
        self.event = torch.cuda.Event()
        self.in_flight = False

    def launch(self, chunk: int, unroll: int) -> None:
        n = min(chunk, self.remaining)
        self.solver.run_graph(n, unroll)
        self.remaining -= n
        self.event.record(self.solver.stream)
        self.in_flight = True

    def idle(self) -> bool:
        """No chunk of this run is in flight on the device."""
        if self.in_flight and self.event.query():
            self.in_flight = False
        return not self.in_flight

    def finite(self) -> bool:
        """The state holds no NaN or infinity (read on the run's own stream)."""
        torch = _torch()
        with torch.cuda.stream(self.solver.stream):
            return bool(torch.isfinite(torch.view_as_real(self.solver.X)).all().item())

    def result(self):
        s = self.solver
        if hasattr(s, "dev"):
            return s.state_to_host()
        s.stream.synchronize()
        return s.state()


class ServingEngine:
    """Continuous-batching request loop with admission by planned device bytes."""

    def __init__(self, budget_bytes: float = 150e9, precision: str = "fp64", chunk: int = 500,
                 unroll: int = 50, max_active: int = 512, keep_results: bool = False, free_batch: int = 32):
        self.free_batch = int(free_batch)
        self.budget = float(budget_bytes)
        self.precision = precision
        self.chunk = int(chunk)
        self.unroll = int(unroll)
        self.max_active = int(max_active)
        self.keep_results = keep_results

    def run(self, requests: list, realtime: bool = True) -> dict:
        """Serve ``requests``: with ``realtime`` a request becomes visible at its arrival time,
        otherwise all arrive at time 0. Returns latency and throughput statistics."""
        torch = _torch()
        queue = sorted(requests, key=lambda r: r.arrival)
        prepared: Prepared | None = None
        active: list[Session] = []
        retired: list[Session] = []     # finished runs whose device memory is not yet released
        nonfinite = 0
        used = 0
        peak_used = 0
        done = []
        steps_done = 0
        peak_active = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if not realtime:
            for r in queue:
                r.arrival = 0.0
        while queue or active or prepared:
            now = time.perf_counter() - t0
            # admission: first come, first served, while the plan fits the budget
            while len(active) < self.max_active:
                if prepared is None:
                    if not queue or queue[0].arrival > now:
                        break
                    prepared = prepare(queue.pop(0), self.precision)
                if prepared.bytes > self.budget:
                    raise MemoryError(f"request {prepared.req.rid} needs {prepared.bytes} bytes, above the "
                                      f"budget of {self.budget:.0f}")
                if used + prepared.bytes > self.budget and retired:
                    used -= self._release(retired)
                if used + prepared.bytes > self.budget:
                    break
                s = Session(prepared, self.precision)
                prepared.req.admitted = time.perf_counter() - t0
                prepared.req.footprint = prepared.bytes
                used += prepared.bytes
                peak_used = max(peak_used, used)
                active.append(s)
                prepared = None
                now = time.perf_counter() - t0
            peak_active = max(peak_active, len(active))
            # advance every run whose last chunk has completed; retire finished runs
            progressed = False
            for s in list(active):
                if not s.idle():
                    continue
                progressed = True
                if s.remaining == 0:
                    s.req.finished = time.perf_counter() - t0
                    if self.keep_results:
                        s.req.result = s.result()
                    nonfinite += 0 if s.finite() else 1
                    steps_done += s.req.steps
                    active.remove(s)
                    retired.append(s)
                    done.append(s.req)
                    continue
                s.launch(self.chunk, self.unroll)
            if len(retired) >= self.free_batch:
                used -= self._release(retired)
            if not progressed:
                wait = 2e-4
                if not active and queue and prepared is None:
                    wait = max(0.0, min(0.01, queue[0].arrival - (time.perf_counter() - t0)))
                time.sleep(wait)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        self._release(retired)
        lat = np.array([r.finished - r.arrival for r in done]) if done else np.zeros(1)
        return dict(requests=len(done), wall_s=wall, steps=steps_done, steps_per_s=steps_done / wall,
                    nonfinite=nonfinite,
                    p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)),
                    peak_active=peak_active, peak_planned_bytes=int(peak_used), budget_bytes=self.budget,
                    by_kind={k: sum(1 for r in done if r.kind == k) for k in ("burgers", "ks", "rb")})

    @staticmethod
    def _release(retired: list) -> int:
        """Free the device memory of finished runs, all at once: releasing device memory waits for
        the whole device, so it is batched rather than done run by run. Returns the planned bytes
        released."""
        n = sum(s.footprint for s in retired)
        retired.clear()
        return n
