"""Serving: a request loop that admits IVP runs of different kinds and resolutions as they arrive
and advances them in shared launches (continuous batching).

Each request asks for ``steps`` IMEX steps of one model (Burgers, Kuramoto-Sivashinsky or 2D
Rayleigh-Benard, each with its own resolution and parameter). Requests of one template at one
resolution and one time step share a *pool*: a stacked problem of a fixed number of slots
(``template.StackedProblem`` for Burgers and Rayleigh-Benard, whose parameter enters L linearly;
``ensemble.FourierEnsemble`` for KS, one period per member), resident on the device with its
state, history ring and factored operators, and advanced by one set of launches per step for every
member (CUDA graphs on the pool's own stream; the pools overlap on the device). The engine

* plans a pool's device bytes before allocating it (``conatus_gb300.memory``) and admits a request
  once it has arrived and a slot of its pool is free, creating the pool when the HBM budget left by
  the pools in flight allows (first come, first served: a request that cannot be placed waits, and
  so do the requests behind it); pools left without members are released when the budget is needed;
* places new members at the next chunk boundary of their pool: their parameters go into the pool's
  operators (refactored once for all the members placed at that boundary), and their first step,
  the lower-order start-up of the reference's ``startup="lower_order"``, runs in a start-up copy of
  the pool, whose state and history then seed the member's slot;
* ends a chunk at every member's last step and at least every 100 steps, checks every member's
  state there and stops a member whose state holds a NaN or an infinity (the reference's
  finite-state check every 100 steps, python/conatus/timestep/run_checks.py:15-20), retiring it
  with that status while the others continue;
* records arrival, admission and completion times: p50/p99 completion latency (completion minus
  arrival) and aggregate steps/s.

Every system of a slot is solved, and every line of its transforms computed, by the same
arithmetic whatever the other slots hold, so a request gives bit for bit the same result served
alone and in the mix. The reference serves nothing: it runs one ``Simulation`` per process
(python/conatus/model/run.py).
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

__all__ = ["Request", "poisson_stream", "pool_key", "Pool", "ServingEngine"]

BURGERS_N = tuple(range(64, 513, 32))     # resolutions with a parameter-linear template
RB_NZ = (32, 48, 64, 80, 96)
SCHEME = "SBDF2"
DT = {"burgers": 1e-4, "ks": 1e-2, "rb": 1e-4}
# slots per pool: about the members a pool of the configured stream holds at once (measured: a
# Burgers resolution sees ~6 requests in flight, a KS size ~20, an RB (Nz, dt) key ~2); every slot
# is computed whether it holds a member or not
POOL_SLOTS = {"burgers": 8, "ks": 32, "rb": 2}
CHECK_EVERY = 100                         # steps between two finite-state checks of a member
RB_LX = 2 * math.pi / 3.117


def time_step(req) -> float:
    """dt of a request: 1e-4 for Burgers, 1e-2 for KS; for RB the largest 1e-4 / 4^k below an
    advective limit, a quarter of the grid spacing Lx/Nx over the free-fall velocity (Ra Pr)^(1/2)
    (thermal-diffusion units, Pr = 1): the explicit advection of SBDF2 at dt = 1e-4 diverges from
    Ra ~ 1e5 up (the reference's own runs blow up), and steps on a 4^-k ladder let requests of
    nearby Ra share a pool."""
    if req.kind == "rb":
        limit = 0.25 * (RB_LX / req.params["Nx"]) / math.sqrt(req.params["Ra"])
        k = max(0, math.ceil(math.log(DT["rb"] / limit, 4)))
        return DT["rb"] * 4.0 ** -k
    return DT[req.kind]


def pool_key(req) -> tuple:
    """Requests with one key share a pool: the template, the resolution and the time step."""
    p = req.params
    if req.kind == "burgers":
        return ("burgers", p["N"], time_step(req))
    if req.kind == "ks":
        return ("ks", p["N"], time_step(req))
    return ("rb", p["Nz"], p["Nx"], time_step(req))


@dataclass
class Request:
    rid: int
    kind: str                     # "burgers" | "ks" | "rb"
    params: dict
    steps: int
    arrival: float                # seconds after the start of the stream
    admitted: float | None = None
    finished: float | None = None
    footprint: int = 0            # planned bytes of the pool it joined
    result: object = None
    status: str = "queued"        # "running", "done", "nonfinite"
    slot: tuple | None = None     # (pool key, slot index)


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


def _pool_problem(key, slots, params=None):
    """(template, stacked problem) of a Burgers / RB pool; every slot at ``params`` (default: the
    template's own parameter values)."""
    if key[0] == "burgers":
        tpl = _template(f"burgers_n{key[1]}_nu")
        sizes = None
    else:
        tpl = _template(f"rb_nz{key[1]}_ra")
        sizes = [key[2]]
    from .template import StackedProblem
    base = params or {k: float(tpl.params[k]) for k in tpl.linear_params}
    return tpl, StackedProblem(tpl, sizes, [dict(base) for _ in range(slots)])


def plan_pool(key, slots: int, precision: str = "fp64") -> int:
    """Planned device bytes of a pool: its solver (state, history, operators, one factor set per
    SBDF order) and the start-up copy's state and history."""
    if key[0] == "ks":
        return 2 * memory.plan_fourier_ensemble([key[1]] * slots, SCHEME)["total"]
    _, S = _pool_problem(key, slots)
    plan = memory.plan_ivp(S, SCHEME, precision, factor_sets=2)
    q = int(SCHEME[-1])
    return int(plan["total"] + (2 + 2 * q) * 16 * S.n_total)


def ks_state(N: int, seed: int, amplitude: float = 0.1, kmax: int = 8) -> np.ndarray:
    """A KS request's initial amplitudes: seeded Fourier amplitudes of size ``amplitude`` for mode
    indices 1..kmax (the KS configuration; one member of ``FourierEnsemble.random_state``)."""
    rng = np.random.default_rng(seed)
    c = np.zeros(N // 2, np.complex128)
    k = min(kmax, N // 2 - 1)
    c[1:k + 1] = amplitude * (rng.standard_normal(k) + 1j * rng.standard_normal(k))
    return c


class Pool:
    """Slots of one pool key, advanced together (see module docstring)."""

    def __init__(self, key, slots: int, precision: str = "fp64", chunk: int = 500, unroll: int = 50):
        torch = _torch()
        self.key, self.slots, self.precision = key, int(slots), precision
        self.chunk, self.unroll = int(chunk), int(unroll)
        self.kind = key[0]
        self.members = [None] * self.slots        # Request per slot
        self.remaining = [0] * self.slots
        self.pending = []                          # (slot, request) placed at the next boundary
        self.dt = key[-1]
        self.footprint = plan_pool(key, self.slots, precision)
        if self.kind == "ks":
            from .ensemble import FourierEnsemble
            N = key[1]
            self.main = FourierEnsemble(_template("ks"), [N] * self.slots, [22.0] * self.slots, scheme=SCHEME,
                                        dt=self.dt, precision=precision)
            self.start = FourierEnsemble(_template("ks"), [N] * self.slots, [22.0] * self.slots, scheme=SCHEME,
                                         dt=self.dt, precision=precision)
            self.main.set_state([np.zeros(N // 2, np.complex128)] * self.slots)
        else:
            from .ivp import DeviceProblem
            self.tpl, self.S = _pool_problem(key, self.slots)
            self.dev = DeviceProblem(self.S, precision, factor_sets=2)
            self.main = IVPSolver(self.S, scheme=SCHEME, dt=self.dt, device_problem=self.dev, check_finite=False)
            self.start = IVPSolver(self.S, scheme=SCHEME, dt=self.dt, device_problem=self.dev, check_finite=False)
            self.main.fork = self.start.fork = False
        for s in (self.main, self.start):
            s.stream.wait_stream(torch.cuda.current_stream())
            s.join = False
        self.event = torch.cuda.Event()
        self.in_flight = False
        self.seeded = False                        # the main solver's history is full

    # ---- bookkeeping
    def free(self) -> int:
        return self.members.count(None) - len(self.pending)

    def empty(self) -> bool:
        return not self.pending and all(m is None for m in self.members)

    def place(self, req) -> None:
        """Reserve a slot for ``req``; it joins at the next chunk boundary."""
        taken = {c for c, _ in self.pending}
        c = next(i for i, m in enumerate(self.members) if m is None and i not in taken)
        self.pending.append((c, req))
        req.slot = (self.key, c)

    def idle(self) -> bool:
        if self.in_flight and self.event.query():
            self.in_flight = False
        return not self.in_flight

    # ---- layout of a slot
    def _slices(self, c):
        """(flat tensor, slice) pairs of slot c in a mode-layout vector of the pool."""
        if self.kind == "ks":
            k = self.key[1] // 2
            return [slice(c * k, (c + 1) * k)]
        out = []
        for bi, b in enumerate(self.S.tpl.buckets):
            ns = self.S._nsys_case[bi]
            o = self.S.offsets[bi] + c * ns * b.n
            out.append(slice(o, o + ns * b.n))
        return out

    def _copy_slot(self, dst, src, c) -> None:
        for sl in self._slices(c):
            dst[sl].copy_(src[sl])

    def _zero_slot(self, dst, c) -> None:
        for sl in self._slices(c):
            dst[sl].zero_()

    def slot_state(self, c):
        """Host copy of slot c's state (per bucket (nsys, n), or the KS member's amplitudes)."""
        x = self.main.X.detach().cpu().numpy()
        if self.kind == "ks":
            return [x[self._slices(c)[0]]]
        return [x[sl].reshape(-1, b.n) for sl, b in zip(self._slices(c), self.S.tpl.buckets)]

    def finite_slots(self) -> np.ndarray:
        """Per slot: its state holds no NaN or infinity (read on the pool's stream, waited for)."""
        torch = _torch()
        with torch.cuda.stream(self.main.stream):
            x = torch.view_as_real(self.main.X)
            if self.kind == "ks":
                ok = torch.isfinite(x.view(self.slots, -1)).all(dim=1)
            else:
                ok = None
                for bi, b in enumerate(self.S.tpl.buckets):
                    o, ns = self.S.offsets[bi], self.S._nsys_case[bi]
                    blk = x[o:o + self.slots * ns * b.n].reshape(self.slots, -1)
                    f = torch.isfinite(blk).all(dim=1)
                    ok = f if ok is None else ok & f
            return ok.cpu().numpy()

    # ---- the chunk boundary
    def boundary(self, now) -> list:
        """At a chunk boundary (pool idle): retire finished members (and diverged ones), then place
        the pending ones. Returns the requests that left."""
        left = []
        if any(m is not None for m in self.members):
            ok = self.finite_slots()
            for c, m in enumerate(self.members):
                if m is None:
                    continue
                if not ok[c] or self.remaining[c] == 0:
                    m.status = "done" if ok[c] else "nonfinite"
                    m.result = self.slot_state(c) if ok[c] else None
                    m.finished = now()
                    left.append(m)
                    self.members[c] = None
                    for v in [self.main.X] + list(self.main.MXh) + list(self.main.Fh):
                        self._zero_slot(v, c)
        if self.pending:
            self._join([c for c, _ in self.pending], [r for _, r in self.pending])
            self.pending = []
        return left

    def _join(self, cs, reqs) -> None:
        torch = _torch()
        main, start = self.main, self.start
        # the members' parameters into the pool's operators (one refactorization for all)
        if self.kind == "ks":
            for c, r in zip(cs, reqs):
                for ens in (main, start):
                    ens.L[c] = r.params["L"]
                    ens._arrs["L"][c] = float(r.params["L"])
        else:
            for c, r in zip(cs, reqs):
                self.S.params[c] = {k: float(r.params[k]) for k in self.S.params[c]}
            self.dev.reset_operators()
            main.operators_changed()
            start.operators_changed()
        # the first step of each new member (lower-order start-up) in the start-up copy
        torch.cuda.current_stream().wait_stream(main.stream)
        X0 = main.X.clone()
        for c, r in zip(cs, reqs):
            st = self._initial(r, c)
            for sl, part in zip(self._slices(c), st):
                X0[sl].copy_(torch.as_tensor(np.ravel(part), device=X0.device))
        if self.kind == "ks":
            start.X.copy_(X0)
            start.head, start.filled = start.order - 1, 0
        else:
            start.set_state(X0)
        start.stream.wait_stream(torch.cuda.current_stream())
        start.run(1) if self.kind == "ks" else start.run_graph(1, wait=False)
        main.stream.wait_stream(start.stream)
        with torch.cuda.stream(main.stream):
            if not self.seeded:
                # the pool's first members: the start-up copy's state and history become the
                # main solver's (history full from here on)
                main.X.copy_(start.X)
                if self.kind == "ks":
                    main.MXh[start.head].copy_(start.MXh[start.head])
                    main.Fh[start.head].copy_(start.Fh[start.head])
                    main.head, main.filled = start.head, 1
                else:
                    main.set_history([start.MXh[start.head]], [start.Fh[start.head]])
                self.seeded = True
            else:
                for c in cs:
                    self._copy_slot(main.X, start.X, c)
                    self._copy_slot(main.MXh[main.head], start.MXh[start.head], c)
                    self._copy_slot(main.Fh[main.head], start.Fh[start.head], c)
        for c, r in zip(cs, reqs):
            self.members[c] = r
            self.remaining[c] = r.steps - 1
            r.status = "running"

    def _initial(self, req, c):
        """Initial state of a request in its slot's layout (seeded by the request id, whatever the
        slot)."""
        if self.kind == "ks":
            return [ks_state(self.key[1], req.rid)]
        P = self.tpl.instantiate(self.S.fourier_sizes or None, None, dict(self.S.params[c]))
        if self.kind == "burgers":
            return W.burgers_state(P)
        return W.rayleigh_benard_state(P, req.rid)

    def launch(self) -> int:
        """Advance every member to the next boundary: the first member's last step, at most
        CHECK_EVERY steps. Returns the steps taken."""
        live = [self.remaining[c] for c, m in enumerate(self.members) if m is not None]
        if not live:
            return 0
        n = min(min(live), self.chunk, CHECK_EVERY)
        if n > 0:
            if self.kind == "ks":
                self.main.run_graph(n, self.unroll)
            else:
                self.main.run_graph(n, self.unroll, wait=False)
        for c, m in enumerate(self.members):
            if m is not None:
                self.remaining[c] -= n
        self.event.record(self.main.stream)
        self.in_flight = True
        return n


class ServingEngine:
    """Continuous-batching request loop over pools, admission by planned device bytes."""

    def __init__(self, budget_bytes: float = 150e9, precision: str = "fp64", chunk: int = 500,
                 unroll: int = 25, slots: dict | None = None, keep_results: bool = False,
                 max_pools: int = 256):
        self.budget = float(budget_bytes)
        self.precision = precision
        self.chunk = int(chunk)
        self.unroll = int(unroll)
        self.slots = dict(POOL_SLOTS, **(slots or {}))
        self.keep_results = keep_results
        self.max_pools = int(max_pools)

    def _new_pool(self, key):
        return Pool(key, self.slots[key[0]], self.precision, self.chunk, self.unroll)

    def run(self, requests: list, realtime: bool = True) -> dict:
        """Serve ``requests``: with ``realtime`` a request becomes visible at its arrival time,
        otherwise all arrive at time 0. Returns latency and throughput statistics."""
        torch = _torch()
        queue = sorted(requests, key=lambda r: r.arrival)
        pools: dict = {}
        used = peak_used = 0
        done, steps_done, nonfinite = [], 0, 0
        peak_members = peak_pools = 0
        budget_waits = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        if not realtime:
            for r in queue:
                r.arrival = 0.0
        while queue or any(not p.empty() for v in pools.values() for p in v):
            # admission: first come, first served
            while queue and queue[0].arrival <= now():
                req = queue[0]
                key = pool_key(req)
                pool = next((p for p in pools.get(key, []) if p.free() > 0), None)
                if pool is None:
                    need = plan_pool(key, self.slots[key[0]], self.precision)
                    if need > self.budget:
                        raise MemoryError(f"request {req.rid}: a pool of {key} needs {need} bytes, above the "
                                          f"budget of {self.budget:.0f}")
                    if used + need > self.budget:
                        used -= self._release_empty(pools)
                    if used + need > self.budget or sum(len(v) for v in pools.values()) >= self.max_pools:
                        budget_waits += 1
                        break
                    pool = self._new_pool(key)
                    pools.setdefault(key, []).append(pool)
                    used += pool.footprint
                    peak_used = max(peak_used, used)
                queue.pop(0)
                pool.place(req)
                req.admitted = now()
                req.footprint = pool.footprint
            members = sum(self.slots[k[0]] - p.free() for k, v in pools.items() for p in v)
            peak_members = max(peak_members, members)
            peak_pools = max(peak_pools, sum(len(v) for v in pools.values()))
            progressed = False
            for plist in pools.values():
                for p in plist:
                    if p.empty() or not p.idle():
                        continue
                    progressed = True
                    for r in p.boundary(now):
                        done.append(r)
                        if r.status == "done":
                            steps_done += r.steps
                        else:
                            nonfinite += 1
                        if not self.keep_results:
                            r.result = None
                    p.launch()
            if not progressed:
                wait = 2e-4
                if queue and all(p.empty() for v in pools.values() for p in v):
                    wait = max(0.0, min(0.01, queue[0].arrival - now()))
                time.sleep(wait)
        torch.cuda.synchronize()
        wall = now()
        lat = np.array([r.finished - r.arrival for r in done]) if done else np.zeros(1)
        return dict(requests=len(done), wall_s=wall, steps=steps_done, steps_per_s=steps_done / wall,
                    nonfinite=nonfinite, p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)),
                    peak_members=peak_members, peak_pools=peak_pools, peak_planned_bytes=int(peak_used),
                    budget_bytes=self.budget, budget_waits=budget_waits,
                    by_kind={k: sum(1 for r in done if r.kind == k) for k in ("burgers", "ks", "rb")})

    @staticmethod
    def _release_empty(pools) -> int:
        """Free the pools left without members (their device memory goes back once the objects
        are dropped). Returns their planned bytes."""
        freed = 0
        for key in list(pools):
            keep = []
            for p in pools[key]:
                if p.empty() and p.idle():
                    freed += p.footprint
                else:
                    keep.append(p)
            if keep:
                pools[key] = keep
            else:
                del pools[key]
        return freed
