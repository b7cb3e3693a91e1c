"""Benchmark of the IMEX step (the reference's IVPSolver SBDF path) on the GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--config channel|rayleigh_benard|burgers] [--precision fp64|fp32]

Default workload: the 3D plane channel 192 x 129 x 192 (Lx = 4 pi, Lz = 2 pi, Re = 4000), SBDF3,
dt = 5e-3, FP64, seeded divergence-free initial perturbation (conatus_gb300.workloads). A step is
one IMEX step of every Fourier mode: M X, the dealiased pseudospectral F, the SBDF right-hand side
and the batched bordered-banded solves. ``value`` is steps/s of the whole job with the state
resident in HBM (CUDA events on the stepping stream, max over ranks); ``e2e`` is the same metric
through the public API with the state copied in from pinned host memory and back out every step.
N > 1 (torchrun): independent replicas, one per GPU (weak scaling, no collective on the path).

``--impl reference`` times the reference algorithm on the host cores instead: the CPU restatement
of the reference's IVPSolver step (oracle/ivp.py), full steps of the same workload, the solves of
every system spread over one process per core.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = {
    "channel": "IMEX steps/s (3D channel 192x129x192, SBDF3)",
    "rayleigh_benard": "IMEX steps/s (2D Rayleigh-Benard 256x64, SBDF2)",
    "burgers": "IMEX steps/s (1D Burgers N=128, SBDF2)",
}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while active. Entering waits
    (at most 5 s) for nvidia-smi's first sample, which is taken before the timed region and left
    out, so that the samples kept cover the whole region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows, self.proc, self.gpu, self.skip = [], None, gpu_index, 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return self
        deadline = time.perf_counter() + 5.0
        while not self.rows and self.proc.poll() is None and time.perf_counter() < deadline:
            time.sleep(0.005)
        self.skip = len(self.rows)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        # the samples taken inside the region (the pre-region one only if the region was shorter
        # than one interval)
        rows = self.rows[self.skip:] or self.rows
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def solve_bytes(dev, fs):
    """Algorithmic bytes of one batched solve launch, band-equivalent (as the reference's band
    kernel reads them): per system the band LU (ldab n), V^T and W (2 r n) and the capacitance LU
    (r r) in the factor precision, pivots (4 n), right-hand side in and solution out (2 n
    complex128); a shared pair's partner reads its primary's factors in the same sweep (the
    reference's SharedFactor), so only its right-hand side and solution count."""
    ef = 8 if dev.precision == "fp32" else 16
    tot = 0
    for h in fs:
        ns, n, r, ldab = h.batch, h.n, h.rank, h.ldab
        if getattr(h, "primary", None) is not None:     # shared pair: the primary's factors, read once
            tot += ns * 32 * n
            continue
        tot += ns * (ef * (ldab * n + 2 * r * n + r * r) + 4 * n + 32 * n)
    return tot


def step_bytes(dev, solver):
    """Algorithmic bytes of one steady step (the model of the hot path's traffic): the solve
    (one launch; the FP32 form: two launches, plus the FP64 residual reading x and the right-hand
    side and writing r), the right-hand side combination ((2q + 1) vectors of the mode layout for
    SBDF-q) and M X (X read, M X written), and F (the state read and the rows written, plus each of
    the n_f factor and n_o output grids written once and read once in the transform precision)."""
    fs = dev.factor(*solver._step_keys()[0])
    vec = 16 * dev.n_total
    b_solve = solve_bytes(dev, fs)
    if dev.precision == "fp32":
        b_solve = 2 * b_solve + 3 * vec
    q = solver.ring
    b_rhs = (2 * q + 1) * vec + 2 * vec
    g = dev.grid
    M_g = max(g["mx"], 1) * max(g["mz"], 1) * max(g["my"], 1)
    s_r = 4 if dev.precision == "fp32" else 8
    nf, no = len(dev.tpl.factors), len(dev.tpl.outputs)
    b_F = 2 * vec + (nf + no) * 2 * M_g * s_r
    return {"solve": b_solve, "rhs_and_MX": b_rhs, "F": b_F, "total": b_solve + b_rhs + b_F}


# DRAM bytes per system of one batched solve launch, from the ncu captures of the channel solve
# (64x129x64; dram__bytes_read.sum + dram__bytes_write.sum): the compact solve reads the union pattern
# of the factors, not the band, and a shared pair's factors once for both systems, so its traffic is
# below the band-equivalent bytes. Per solve kernel: the windowed solve adds its scratch round trip
# (mostly absorbed by L2)
TRAFFIC_PER_SYSTEM = {
    ("channel", "fp64", "k_solve_compact_multi"): ((174.600192 + 3.016192) * 1e6 / 1985,
                                                   "profiles/k_solve_compact_multi_channel64x129x64_fp64.md"),
    ("channel", "fp64", "k_solve_window_multi"): ((177.924352 + 15.470848) * 1e6 / 1985,
                                                  "profiles/k_solve_window_multi_lanes8_channel64x129x64_fp64.md"),
    # the FP32 form solves in two groups: the captured launch is the group of 1024 paired systems
    ("channel", "fp32", "k_solve_compact_multi"): ((47.700736 + 0.423936) * 1e6 / 1024,
                                                   "profiles/k_solve_compact_multi_channel64x129x64_fp32.md"),
    ("channel", "fp32", "k_solve_window_multi"): ((47.577856 + 0.329984) * 1e6 / 1024,
                                                  "profiles/k_solve_window_multi_channel64x129x64_fp32.md"),
}


def solve_kernel(sched: int) -> str:
    """The kernel that runs solve schedule ``sched`` (-1: the band kernel)."""
    from conatus_gb300 import autotune
    if sched is None or sched < 0:
        return "k_solve"
    if sched in autotune.windowed_schedules():
        return "k_solve_window_multi"
    if sched in autotune.partitioned_schedules():
        return "k_solve_part"
    if sched in autotune.split_schedules():
        return "k_solve_split_multi"
    return "k_solve_compact_multi"


# DRAM bytes of the F pipeline's x backward real transform on the channel 64x129x64 (ncu: read +
# write; it reads the 9 z-groups, 32 modes x 19200 columns, and writes the 12 factor fields, 96
# points x 19200 columns) and the algorithmic bytes of that launch; the full launch's traffic is
# taken in the same proportion to its algorithmic bytes (the transform streams its fields once)
RFFT_TRAFFIC = ((95.617024 + 126.273024) * 1e6, 9 * 19200 * 32 * 16 + 12 * 19200 * 96 * 8,
                "profiles/k_rfft_axis_channel64x129x64_fp64.md")
FP64_NOMINAL_TFLOPS = 1.25     # GB300 FP64 (2 DFMA per clock per SM): nominal


def fp64_peak(stream, reps=3):
    """FP64 rate measured here: the library's DFMA loop (cng_dfma_probe, 8 independent chains per
    thread on every SM), best of ``reps`` CUDA-event timings, TFLOP/s (a fused multiply-add is two
    flops)."""
    import ctypes
    import torch
    from conatus_gb300._lib import call
    sink = torch.zeros(1, dtype=torch.float64, device="cuda")
    fl = ctypes.c_double()
    sh = stream.cuda_stream
    call("cng_dfma_probe", 2000, 8, sink.data_ptr(), ctypes.byref(fl), sh)      # warm-up
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call("cng_dfma_probe", 20000, 8, sink.data_ptr(), ctypes.byref(fl), sh)
        e1.record(stream)
        e1.synchronize()
        t = fl.value / (e0.elapsed_time(e1) / 1e3) / 1e12
        best = t if best is None else max(best, t)
    return best


def rfft_roofline(dev, stream, hbm_peak, peak_kind, reps=5):
    """Roofline of the FP64 step's dominant kernel: the x backward real transform of every factor
    field (k_rfft_axis<double>), launched alone through cng_rfft_axis with the step's shapes.
    Algorithmic bytes: K complex modes read and L reals written per column and field. FLOPs: the
    conventional 2.5 L log2 L per real transform of length L. The kernel is bound by the FP64 pipe
    (GB300 issues FP64 at 1/64 of the FP32 rate), so its HBM fraction is low by construction; the
    FP64 fraction is against the FP64 rate measured in the same run (cng_dfma_probe)."""
    import math
    import torch
    from conatus_gb300._lib import call
    g = dev.grid
    nf = len(dev.tpl.factors) * int(getattr(dev.P, "ncase", 1))
    K = dev.P.fourier_sizes[0] // 2
    inner = max(g["mz"], 1) * max(g["my"], 1)
    L = g["mx"]
    x = torch.zeros(nf * K * inner, dtype=torch.complex128, device="cuda")
    y = torch.zeros(nf * L * inner, dtype=torch.float64, device="cuda")
    x.real.normal_()
    x.imag.normal_()
    sh = stream.cuda_stream
    torch.cuda.synchronize()
    call("cng_rfft_axis", 0, x.data_ptr(), y.data_ptr(), nf, inner, K, L, sh)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        call("cng_rfft_axis", 0, x.data_ptr(), y.data_ptr(), nf, inner, K, L, sh)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nbytes = nf * inner * (16 * K + 8 * L)
    flops = nf * inner * 2.5 * L * math.log2(L)
    achieved = nbytes / (ms / 1e3) / 1e9
    small_traffic, small_bytes, src = RFFT_TRAFFIC
    traffic = small_traffic * nbytes / small_bytes if small_traffic else None
    del x, y
    peak64 = fp64_peak(stream)
    return {"kernel": f"k_rfft_axis<double> (x backward, {nf} factor fields, {K} modes -> {L} points, "
                      f"{inner} columns), launched alone",
            "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
            "traffic": traffic,
            "traffic_source": (src + " (traffic / algorithmic bytes of the F pipeline's launch, small case)")
            if traffic else None,
            "algorithmic_bytes": nbytes, "launch_ms": ms, "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "binding_roof": {"pipe": "fp64", "achieved_tflops": flops / (ms / 1e3) / 1e12,
                             "peak_tflops": peak64,
                             "peak_kind": "measured (cng_dfma_probe: FP64 fused multiply-add loop, this run)",
                             "nominal_tflops": FP64_NOMINAL_TFLOPS,
                             "frac": flops / (ms / 1e3) / 1e12 / peak64,
                             "flops": flops, "flop_count": "2.5 L log2 L per real transform"}}


def max_over_ranks(x: float) -> float:
    """The largest x over the ranks of the process group (x itself without one): the timed region
    of the slowest replica. NCCL reduces on the GPU, gloo on the host."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, steps: int, ms: float) -> float:
    """Whole-job steps/s of ``world`` independent replicas of ``steps`` steps each, timed by the
    slowest (weak scaling: every replica does the full workload)."""
    return world * steps / (ms / 1e3)


L2_BYTES = 129e6      # GB300 L2


def _l2_note(P, cfg, precision):
    """Whether the timed steps stream from HBM: the planned device bytes of the run against L2."""
    from conatus_gb300 import memory
    nbytes = memory.plan_ivp(P, cfg["scheme"], precision)["total"]
    if nbytes > L2_BYTES:
        return f"inputs larger than L2 (state, history and factors: {nbytes / 1e9:.2f} GB planned)"
    return (f"fits in L2 ({nbytes / 1e6:.1f} MB planned; not flushed between steps: the steps of a "
            f"small problem run from L2 in use too)")


def workload_config(args, P, ws):
    """The ``config`` of both arms' lines: the workload, its size, the replicas and whether the
    timed steps stream from HBM (the same dict for the GB300 arm and the reference arm)."""
    cfg = args.cfg
    return {"workload": f"{args.config} {P.fourier_sizes} x {P.tpl.ncheb} {cfg['scheme']} dt={cfg['dt']}",
            "real_unknowns": P.real_unknowns(), "systems": int(sum(P.nsys)),
            "parallelism": f"replicas x{ws}" if ws > 1 else "1 replica",
            "l2": _l2_note(P, cfg, args.precision)}


def run_gpu(args):
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import DeviceProblem, IVPSolver
    cfg = args.cfg
    P = W.problem(args.config, args.fourier)
    C0 = W.initial_state(args.config, P, seed=rank)
    dp = DeviceProblem(P, args.precision)
    dp.partitioned = dp.partitioned or args.partitioned
    solver = IVPSolver(P, scheme=cfg["scheme"], dt=cfg["dt"], precision=args.precision, device_problem=dp)
    dev = solver.dev
    solver.set_state(C0)
    solver.run_graph(max(args.warmup, solver.ring))            # start-up, capture, warm-up
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- timed region: K steps, state resident in HBM
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed_steps")       # the profiles' launch lists filter on it
        e0.record(solver.stream)
        solver.run_graph(args.steps)
        e1.record(solver.stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1))
    ms_step = ms / args.steps
    value = replica_throughput(ws, args.steps, ms)
    finite = bool(torch.isfinite(torch.view_as_real(solver.X)).all().item())

    # ---- per-kernel timing (same stream, CUDA events): one batched solve launch, and F
    s = solver.stream
    reps = 5
    fs = dev.factor(*solver._step_keys()[0])
    R = dev.zeros()
    R.copy_(solver.X)
    X2 = dev.zeros()
    torch.cuda.synchronize()
    ts = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ts[0].record(s)
    for _ in range(reps):
        dev.solve_launch(fs, R, X2, s)
    ts[1].record(s)
    for _ in range(reps):
        dev.F(solver.X, R, s)
    ts[2].record(s)
    torch.cuda.synchronize()
    solve_ms = ts[0].elapsed_time(ts[1]) / reps
    f_ms = ts[1].elapsed_time(ts[2]) / reps
    hbm_peak, peak_kind = measured_peaks()
    sb = solve_bytes(dev, fs)
    nsys = sum(h.batch for h in fs)
    kname = solve_kernel(getattr(next(h for h in fs if h.h is not None), "schedule", 0))
    tr = TRAFFIC_PER_SYSTEM.get((args.config, args.precision, kname)) if args.fourier is None else None
    solve_roof = {"kernel": kname + " (batched bordered-banded solve, all buckets in one launch)",
            "bound": "hbm", "achieved": sb / (solve_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
            "frac": sb / (solve_ms / 1e3) / 1e9 / hbm_peak,
            "traffic": tr[0] * nsys if tr else None,
            "traffic_source": (tr[1] + " (bytes per system x systems)") if tr else None,
            "algorithmic_bytes": sb, "launch_ms": solve_ms, "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "F_ms": f_ms}
    # the dominant kernel: the batched solve (two launches per step in the FP32 form), unless the
    # x backward real transform takes longer (the FP64 channel: FP64-pipe bound)
    roof = solve_roof
    if args.precision == "fp64" and dev.d >= 1:
        rf = rfft_roofline(dev, s, hbm_peak, peak_kind)
        if rf["launch_ms"] > solve_ms:
            roof = rf
            roof["F_ms"] = f_ms
    sbytes = step_bytes(dev, solver)
    step_roof = {"bytes_per_step": sbytes, "achieved": sbytes["total"] / (ms_step / 1e3) / 1e9,
                 "unit": "GB/s", "frac": sbytes["total"] / (ms_step / 1e3) / 1e9 / hbm_peak}

    # ---- end to end through the public API: host state in and out every step
    import torch as _t
    host_in = _t.empty(dev.n_total, dtype=_t.complex128, pin_memory=True)
    host_out = _t.empty(dev.n_total, dtype=_t.complex128, pin_memory=True)
    host_in.copy_(solver.X.cpu())
    ke = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke):
        solver.step_host(host_in, host_out)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / ke
    nbytes = dev.n_total * 16
    out = {
        "metric": METRIC[args.config] + (" FP32 form" if args.precision == "fp32" else " plain FP64") +
                  (", partitioned solve allowed" if args.partitioned else ""),
        "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded initial state of the configuration, conatus_gb300.workloads)",
        "config": workload_config(args, P, ws),
        "details": {"grid": dev.grid, "state_finite": finite,
                    "solve_schedule": _schedule_summary(dev),
                    "rhs_transforms": ({"chosen": min(dev.rhs_tuning, key=lambda k: dev.rhs_tuning[k] or 0),
                                        "ms_per_F": {k: (round(v, 4) if v else None)
                                                     for k, v in dev.rhs_tuning.items()}}
                                       if dev.rhs_tuning else None)},
        "mode_updates_per_s": value * P.real_unknowns(),
        "roofline": roof,
        "solve_roofline": solve_roof,
        "step_roofline": step_roof,
        "e2e": {"value": ws / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "gpu_launches": solver.launches_per_step() * args.steps,
        "clocks": clk.summary(),
    }
    if args.precision == "fp32" and rank == 0 and args.error_steps > 0:
        out["error_vs_fp64"] = mixed_error(P, C0, cfg, args.error_steps)
    if args.precision == "fp64" and args.config == "channel" and ws == 1 and not args.no_forms:
        # the precision form beside the drop-in, on the same workload and GPU
        del solver, dev, R, X2
        torch.cuda.empty_cache()
        out["forms"] = {"fp32": form_fp32(P, C0, cfg, args)}
    if args.config == "channel" and ws == 1 and not args.no_forms:
        out["subrecords"] = subrecords(args)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, P, C0)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def subrecords(args):
    """The other configurations, compact and time-bounded, beside the default line: the serving
    stream (100 requests at 200/s, steps U[1000, 20000]; FP64 and the FP32 form under the 150 GB
    budget, FP64 under a 1.5 GB budget that binds), RB 256x64 and Burgers in FP64 with and without
    the partitioned solve, the KS ensemble (4096 members, 500 steps) and the RB ensemble (1024 cases
    of three Nz, 50 steps) in the FP32 form."""
    import copy
    import torch
    out = {}
    # the configured 150 GB budget (the stream's pools plan about 4-8 GB together: it does not
    # bind), and the same FP64 stream under a 1.5 GB budget (about two of its largest pools), where
    # admission waits for pools to empty
    for name, prec, budget in (("serving_fp64", "fp64", 150e9), ("serving_fp32", "fp32", 150e9),
                               ("serving_fp64_budget_1.5gb", "fp64", 1.5e9)):
        a = copy.copy(args)
        a.precision, a.chunk, a.unroll = prec, 500, 25
        rec = serving_record(a, requests=100, rate=200.0, steps=(1000, 20000), budget=budget)
        st = rec["serving"]
        out[name] = {"metric": rec["metric"], "value": rec["value"], "unit": "steps/s",
                     "dtype": rec["dtype"], "latency_s": rec["latency_s"],
                     "requests": st["requests"], "steps": st["steps"], "wall_s": st["wall_s"],
                     "nonfinite": st["nonfinite"], "peak_pools": st["peak_pools"],
                     "peak_members": st["peak_members"], "budget_waits": st["budget_waits"],
                     "peak_planned_gb": st["peak_planned_bytes"] / 1e9, "budget_gb": budget / 1e9,
                     "workload": rec["config"]["workload"]}
        torch.cuda.empty_cache()
    out["small_fp64_partitioned"] = partitioned_record()
    torch.cuda.empty_cache()
    for name, fn, members, steps in (("ks_ensemble", ks_ensemble_record, 4096, 500),
                                     ("rb_ensemble", rb_ensemble_record, 1024, 50)):
        a = copy.copy(args)
        a.precision, a.members, a.steps, a.warmup, a.unroll = "fp32", members, steps, 3, 25
        rec = fn(a)
        out[name] = {k: rec[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "dtype",
                                          "member_steps_per_s", "mode_updates_per_s") if k in rec}
        out[name]["workload"] = rec["config"]["workload"]
        if "launches_per_step" in rec["config"]:
            out[name]["launches_per_step"] = rec["config"]["launches_per_step"]
        torch.cuda.empty_cache()
    return out


def partitioned_record(steps=100, warmup=5):
    """RB 256x64 (SBDF2 and RK443) and Burgers N=128 in FP64, graph-replayed steps with the tuner's
    sequential-sweep schedules and with the partitioned solve allowed, from the same state: steps/s
    of each and the relative difference of the two final states (the partitioned solve's rounding).
    100 steps: RB's configured state grows too fast to stay finite past about 200 steps at dt=1e-4."""
    import torch
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import DeviceProblem, IVPSolver
    out = {}
    for name, config, scheme in (("rayleigh_benard_sbdf2", "rayleigh_benard", None),
                                 ("rayleigh_benard_rk443", "rayleigh_benard", "RK443"),
                                 ("burgers_sbdf2", "burgers", None)):
        cfg = W.CONFIGS[config]
        P = W.problem(config)
        C0 = W.initial_state(config, P, seed=0)
        rec, X = {}, []
        for part in (False, True):
            dev = DeviceProblem(P, "fp64")
            dev.partitioned = part
            s = IVPSolver(P, scheme=scheme or cfg["scheme"], dt=cfg["dt"], device_problem=dev)
            s.set_state(C0)
            s.run_graph(max(warmup, s.ring))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s.stream)
            s.run_graph(steps)
            e1.record(s.stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            key = "partitioned" if part else "sequential"
            rec[key] = {"steps_per_s": 1e3 / ms, "ms_per_step": ms, "solve_schedule": _schedule_summary(dev)}
            X.append(s.X.clone())
            del s, dev
        rec["state_rel_diff"] = float(torch.linalg.vector_norm(X[1] - X[0]) / torch.linalg.vector_norm(X[0]))
        rec["speedup"] = rec["sequential"]["ms_per_step"] / rec["partitioned"]["ms_per_step"]
        rec["steps"] = steps
        out[name] = rec
        torch.cuda.empty_cache()
    return out


def form_fp32(P, C0, cfg, args):
    """The FP32 form (FP32 F and solves, FP64 refinement, state and history) on the workload of the
    FP64 line: steps/s over the same number of graph-launched steps (CUDA events on its stream) and
    its error per field against the FP64 form after ``error_steps`` steps."""
    import torch
    from conatus_gb300.ivp import IVPSolver
    s = IVPSolver(P, scheme=cfg["scheme"], dt=cfg["dt"], precision="fp32")
    s.set_state(C0)
    s.run_graph(max(args.warmup, s.ring))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s.stream)
    s.run_graph(args.steps)
    e1.record(s.stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    res = {"metric": METRIC[args.config] + " FP32 form", "value": args.steps / (ms / 1e3), "unit": "steps/s",
           "ms_per_step": ms / args.steps, "steps": args.steps, "dtype": "f32+f64",
           "gpu_launches": s.launches_per_step() * args.steps}
    # the whole step's algorithmic bytes against the measured HBM rate
    hbm_peak, peak_kind = measured_peaks()
    sbytes = step_bytes(s.dev, s)
    gbs = sbytes["total"] / (ms / args.steps / 1e3) / 1e9
    res["step_roofline"] = {"bytes_per_step": sbytes, "achieved": gbs, "unit": "GB/s", "peak": hbm_peak,
                            "frac": gbs / hbm_peak, "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"}
    res["solve_schedule"] = _schedule_summary(s.dev)
    del s
    torch.cuda.empty_cache()
    if args.error_steps > 0:
        res["error_vs_fp64"] = mixed_error(P, C0, cfg, args.error_steps)
    return res


def _schedule_summary(dev):
    """The solve schedule the autotuner kept (-1: band kernel; k >= 0: compact schedule k) and the
    time per solve it measured for each candidate."""
    from conatus_gb300 import autotune
    cache = autotune.cache()
    for fs in reversed(list(dev._factors.values())):          # the problem's own factor sets
        hit = cache.get(autotune._signature(dev, fs))
        if hit:
            best, times = hit
            return {"chosen": best, "ms_per_solve": {str(k): round(v, 4) for k, v in times.items()}}
    return None


def mixed_error(P, C0, cfg, steps, marks=5):
    """Relative L2 error per field of the mixed form against the plain FP64 form (which matches the
    reference's FP64 CPU path step by step) after ``steps`` steps from the same state, and its
    history at ``marks`` evenly spaced steps (the error at the end of the run is ``max``)."""
    import torch
    from conatus_gb300.ivp import IVPSolver
    at = sorted({max(1, round(steps * (k + 1) / marks)) for k in range(marks)})
    res = {}
    for prec in ("fp64", "fp32"):
        s = IVPSolver(P, scheme=cfg["scheme"], dt=cfg["dt"], precision=prec)
        s.set_state(C0)
        res[prec], done = {}, 0
        for m in at:
            s.run_graph(m - done)
            done = m
            torch.cuda.synchronize()
            res[prec][m] = s.dev.to_host(s.X)
        del s
        torch.cuda.empty_cache()

    def errs(a, b):
        out = {}
        for v, var in enumerate(P.tpl.variables):
            if var["name"].startswith("tau"):
                continue
            num = den = 0.0
            for bi, bk in enumerate(P.tpl.buckets):
                sel = bk.col[:, 0] == v
                num += float(np.sum(np.abs(a[bi][:, sel] - b[bi][:, sel]) ** 2))
                den += float(np.sum(np.abs(b[bi][:, sel]) ** 2))
            out[var["name"]] = (num / den) ** 0.5 if den else 0.0
        return out

    hist = {m: errs(res["fp32"][m], res["fp64"][m]) for m in at}
    final = hist[at[-1]]
    return {"steps": steps, "relative_l2": final, "max": max(final.values()) if final else 0.0,
            "history": {str(m): {k: float(f"{v:.3e}") for k, v in e.items()} for m, e in hist.items()}}


def _host_cores():
    import multiprocessing
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else multiprocessing.cpu_count()


def cpu_baseline(args, P, C0, steps=1, warmup=1):
    """The oracle (CPU restatement of the reference's step) on the host cores: full steps (F, M X,
    right-hand side and the solves of every system, spread over one process per core), after the
    untimed factorization and one untimed step."""
    from oracle.ivp import ParallelStepper
    cores = _host_cores()
    cfg = args.cfg
    st = ParallelStepper(P, int(cfg["scheme"][-1]), cfg["dt"], workers=cores)
    try:
        t_step, desc = st.time_steps(C0, steps, warmup=warmup)
    finally:
        st.close()
    return {"value": 1.0 / t_step, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": desc}


def serving_record(args, requests=None, rate=None, steps=None, budget=150e9):
    """Serve a seeded Poisson stream (conatus_gb300.serving.ServingEngine: pools of requests of one
    template, resolution and step advanced by shared launches, admission by planned bytes under the
    HBM budget) and summarize it: served steps/s, p50/p99 completion latency, pools and members in
    flight. A short warm stream first (templates, twiddles, the autotuner's schedules)."""
    from conatus_gb300 import serving
    requests = requests or args.requests
    rate = rate or args.rate
    lo, hi = steps or args.serve_steps
    warm = serving.poisson_stream(24, rate=1e4, seed=1000, steps=(40, 60))
    serving.ServingEngine(precision=args.precision).run(warm, realtime=False)
    reqs = serving.poisson_stream(requests, rate=rate, seed=0, steps=(lo, hi))
    eng = serving.ServingEngine(budget_bytes=budget, precision=args.precision, chunk=args.chunk,
                                unroll=args.unroll)
    with ClockSampler(0) as clk:
        st = eng.run(reqs, realtime=True)
    return {"metric": "served IMEX steps/s (Poisson mix Burgers/KS/RB, rate %g/s)" % rate,
            "value": st["steps_per_s"], "unit": "steps/s", "requests": st["requests"],
            "steps": st["steps"], "wall_s": st["wall_s"],
            "latency_s": {"p50": st["p50_s"], "p99": st["p99_s"]},
            "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "config": {"workload": f"serving {requests} requests at {rate:g}/s, steps U[{lo},{hi}], SBDF2, "
                                   "Burgers N 64..512 / KS N 64..256 / RB Nz 32..96 Nx 4Nz",
                       "budget_gb": budget / 1e9, "chunk": args.chunk, "unroll": args.unroll,
                       "slots": serving.POOL_SLOTS},
            "serving": st, "clocks": clk.summary()}


def run_serving(args):
    """The serving configuration: a seeded Poisson stream (rate 200/s) of Burgers / KS / RB requests
    served by conatus_gb300.serving.ServingEngine with a 150 GB admission budget."""
    import torch
    torch.cuda.set_device(0)
    rec = serving_record(args)
    out = {"metric": rec["metric"], "value": rec["value"], "unit": "steps/s", "n_gpus": 1,
           "steps": rec["steps"], "warmup": 24, "ms_per_step": 1e3 / max(rec["value"], 1e-30),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": rec["dtype"],
           "data": "synthetic (seeded request stream and initial states)", "config": rec["config"],
           "latency_s": rec["latency_s"], "serving": rec["serving"], "clocks": rec["clocks"]}
    print(json.dumps(out), flush=True)


def run_ks_ensemble(args):
    """The KS ensemble line (see ``ks_ensemble_record``)."""
    import torch
    torch.cuda.set_device(0)
    print(json.dumps(ks_ensemble_record(args)), flush=True)


def ks_ensemble_record(args):
    """The KS ensemble: 4096 members (L ~ U[22, 100], N = next power of two >= 2L), SBDF2, dt = 0.01,
    one fused launch per step replayed as CUDA graphs."""
    import torch
    from conatus_gb300 import workloads as W
    from conatus_gb300.ensemble import FourierEnsemble, ks_members
    N, L = ks_members(args.members, seed=0)
    ens = FourierEnsemble(W.load_template("ks"), N, L, scheme="SBDF2", dt=0.01, precision=args.precision)
    ens.set_state(ens.random_state(seed=0))
    ens.run_graph(max(args.warmup, 3), args.unroll)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(ens.stream)
        ens.run_graph(args.steps, args.unroll)
        e1.record(ens.stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    value = args.steps / (ms / 1e3)
    x = np.concatenate(ens.state())
    out = {"metric": f"ensemble steps/s ({args.members} KS members, SBDF2)", "value": value, "unit": "steps/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64" if args.precision == "fp64" else "f32+f64",
           "data": "synthetic (seeded periods and initial Fourier amplitudes)",
           "config": {"workload": f"KS ensemble {args.members} members N in 64..256, dt=0.01",
                      "modes": int(ens.n_total), "unroll": args.unroll,
                      "l2": "fits in L2 (the ensemble state is a few MB)",
                      "state_finite": bool(np.all(np.isfinite(x)))},
           "member_steps_per_s": value * args.members, "mode_updates_per_s": value * ens.mode_updates(),
           "gpu_launches": args.steps, "clocks": clk.summary()}
    return out


def run_rb_ensemble(args):
    """The RB ensemble line (see ``rb_ensemble_record``)."""
    import torch
    torch.cuda.set_device(0)
    print(json.dumps(rb_ensemble_record(args)), flush=True)


def rb_ensemble_record(args):
    """The RB ensemble: ``--members`` 2D Rayleigh-Benard cases (default 1024), Nz uniform in {32, 48,
    64}, Nx = 4 Nz, Ra log-uniform in [1e4, 1e7], Pr = 1, seeded noise 1e-3. The cases of one Nz are
    stacked (StackedProblem) and the three stacks advanced as one GroupedProblem: every kernel of a
    step is one launch for all 1024 cases (grouped F stages over the three grid sizes, grouped M X,
    one solve launch over every bucket), steps replayed as CUDA graphs. SBDF2 with one dt for all:
    the advective limit of the most restrictive case (a quarter of Lx/Nx over sqrt(Ra), at most
    1e-4)."""
    import math
    import torch
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import IVPSolver
    from conatus_gb300.template import GroupedProblem, StackedProblem
    rng = np.random.default_rng(0)
    nzs = (32, 48, 64)
    nz = rng.choice(nzs, args.members)
    ra = 10 ** rng.uniform(4, 7, args.members)
    lx = 2 * math.pi / 3.117
    stacks, states, info = [], [], []
    dt = 1e-4
    for n in nzs:
        idx = np.nonzero(nz == n)[0]
        if idx.size == 0:
            continue
        tpl = W.load_template(f"rb_nz{n}_ra")
        S = StackedProblem(tpl, [4 * n], [{"Ra": float(ra[i])} for i in idx])
        states.append(S.stack_states([W.rayleigh_benard_state(tpl.instantiate([4 * n], None, {"Ra": float(ra[i])}),
                                                               seed=int(i)) for i in idx]))
        dt = min(dt, 0.25 * (lx / (4 * n)) / math.sqrt(float(ra[idx].max())))
        stacks.append(S)
        info.append({"Nz": n, "Nx": 4 * n, "cases": int(idx.size), "systems": int(sum(S.nsys)),
                     "real_unknowns": S.real_unknowns()})
    G = GroupedProblem(stacks)
    sv = IVPSolver(G, scheme="SBDF2", dt=dt, precision=args.precision, factor_sets=1)
    sv.set_state(G.stack_states(states))
    sv.run_graph(max(args.warmup, 3), args.unroll)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        torch.cuda.nvtx.range_push("timed_steps")               # the launch list filters on it
        e0.record(sv.stream)
        sv.run_graph(args.steps, args.unroll, wait=False)       # the finite check is read below
        e1.record(sv.stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    ms = e0.elapsed_time(e1)
    value = args.steps / (ms / 1e3)
    finite = bool(torch.isfinite(torch.view_as_real(sv.X)).all().item())
    nu = sum(g["real_unknowns"] for g in info)
    out = {"metric": f"ensemble steps/s ({args.members} RB 2D cases, SBDF2)", "value": value, "unit": "steps/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64" if args.precision == "fp64" else "f32+f64",
           "data": "synthetic (seeded Nz, Ra and initial noise)",
           "config": {"workload": f"RB 2D ensemble, {args.members} cases, Nz in {{32, 48, 64}}, Nx = 4 Nz, "
                                  "Ra log-uniform [1e4, 1e7]", "groups": info, "dt": dt, "unroll": args.unroll,
                      "state_finite": finite, "launches_per_step": sv.launches_per_step(),
                      "one_launch_per_kernel": "grouped: every kernel of the step is one launch for all groups",
                      "l2": "inputs larger than L2 (factors of every case)"},
           "member_steps_per_s": value * args.members, "mode_updates_per_s": value * nu,
           "gpu_launches": sv.launches_per_step() * args.steps, "clocks": clk.summary()}
    return out


def run_reference(args):
    """The reference arm: the oracle's restatement of the reference's CPU step (the reference
    cannot run on the GPU host: its core needs nanobind and conda LAPACK, its GPU path CuPy) on
    every host core, ``args.warmup`` untimed and ``args.steps`` timed full steps of the workload."""
    ws, rank, local = _dist()
    if rank != 0:
        return
    from conatus_gb300 import workloads as W
    from oracle.ivp import ParallelStepper
    P = W.problem(args.config)
    C0 = W.initial_state(args.config, P, seed=0)
    cores = _host_cores()
    cfg = args.cfg
    st = ParallelStepper(P, int(cfg["scheme"][-1]), cfg["dt"], workers=cores)
    try:
        t_step, desc = st.time_steps(C0, args.steps, warmup=args.warmup)
    finally:
        st.close()
    value = 1.0 / t_step
    out = {"impl": "reference", "metric": METRIC[args.config] + " plain FP64", "value": value,
           "unit": "steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (seeded initial state of the configuration, conatus_gb300.workloads)",
           "config": workload_config(args, P, ws),
           "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port", "sample": desc},
           "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="channel", choices=list(METRIC) + ["serving", "ks_ensemble", "rb_ensemble"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--scheme", default=None,
                    help="IMEX scheme instead of the configuration's (e.g. RK443: the reference's published "
                         "Rayleigh-Benard case); the CPU baseline times SBDF schemes only")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--partitioned", action="store_true",
                    help="FP64: let the solve tuner take the partitioned solve of small batches (faster "
                         "on RB 256x64 and Burgers; residuals up to about 15x the sequential sweeps')")
    ap.add_argument("--no-forms", action="store_true", help="channel FP64: skip the FP32 form's line")
    ap.add_argument("--error-steps", type=int, default=None,
                    help="steps of the FP32 form's error run (default: the configuration's length)")
    ap.add_argument("--fourier", type=int, nargs="*", default=None,
                    help="Fourier sizes overriding the configuration's (small cases for profiling)")
    ap.add_argument("--requests", type=int, default=200, help="serving: requests in the stream")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: arrivals per second")
    ap.add_argument("--serve-steps", type=int, nargs=2, default=[1000, 20000], help="serving: step range")
    ap.add_argument("--chunk", type=int, default=500, help="serving: most steps per scheduling chunk")
    ap.add_argument("--unroll", type=int, default=25, help="steps per CUDA graph (serving, ensemble)")
    ap.add_argument("--members", type=int, default=None, help="ensembles: members (KS 4096, RB 1024)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.members is None:
        args.members = 1024 if args.config == "rb_ensemble" else 4096
    from conatus_gb300 import workloads as W
    if args.config in ("serving", "ks_ensemble", "rb_ensemble"):
        if args.impl == "reference":
            ws, rank, _ = _dist()
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": f"{args.config}: the reference has no "
                                  "GPU serving or ensemble path; its CPU step is timed on the channel"}))
            return
        {"serving": run_serving, "ks_ensemble": run_ks_ensemble, "rb_ensemble": run_rb_ensemble}[args.config](args)
        return
    args.cfg = dict(W.CONFIGS[args.config])
    if args.scheme:
        if args.scheme != args.cfg["scheme"]:
            METRIC[args.config] = METRIC[args.config].replace(args.cfg["scheme"], args.scheme)
            args.no_cpu_baseline = args.no_cpu_baseline or not args.scheme.startswith("SBDF")
        args.cfg["scheme"] = args.scheme
    if args.error_steps is None:
        args.error_steps = args.cfg.get("finite_steps", args.cfg["steps"])
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
