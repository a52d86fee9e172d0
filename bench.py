#!/usr/bin/env python
"""Benchmark of the Lagrangian-Eulerian interaction hot path on GB300.

Metric: spread + interpolate markers/s (one step = bin the markers, spread
their forces onto the staggered grid, interpolate the staggered velocity
back onto them).  Headline workload: 2,000,000 markers (64 helical fibres
packed in a 0.2^3 sub-box + 400k uniform) on a 256^3 periodic staggered
grid, IB_4 kernel, mixed precision (FP32 values, FP64 positions / indices /
kernel arguments, double-FP32 spread accumulation).  The plain FP64 form on
the same workload, the error against it, the CPU baseline, the end-to-end
rate with host buffers and the roofline of the dominant kernel are reported
on the same JSON line, and nested objects carry the other measured
configurations: ``ib6`` (the same workload with IB_6), ``batched`` (512
independent 2D problems, one CUDA graph per step, autotuned), ``serving``
(Poisson request stream over resident simulations, p50/p99 latency),
``fortran_abi`` (the reference's Fortran entry points with host arrays) and
``kernels`` (IB_3, PIECEWISE_CUBIC and BSPLINE_4 on the 2M-marker workload).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload all|helices|batched|serving] [--kernel K]
                  [--setting k=v,...] [--tune]

The helices workload runs with the plan setting recorded in
profiles/traffic.json (the autotuner's choice, profiled with ncu there, so
that roofline.traffic describes the benched schedule); --tune re-runs the
autotuner instead, --setting fixes another setting.  The batched workload is
always autotuned (tile shape and knobs), as its configuration asks.

Multi-GPU: replicas only (each rank runs the whole workload on its GPU,
value = sum over ranks, "scaling": "weak").
"""

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "spread+interp markers/s"
UNIT = "markers/s"
KERNEL_WIDTHS = {"IB_3": 3, "IB_4": 4, "IB_6": 6, "PIECEWISE_CUBIC": 4, "BSPLINE_4": 4, "PIECEWISE_LINEAR": 2}
N_GRID = 256
DTYPE = "mixed: f32 values, f64 positions/indices, double-f32 accumulation"
TRAFFIC = os.path.join(ROOT, "profiles", "traffic.json")


def helices_workload(kernel):
    return "helices64x25k+uniform400k_256cube_" + kernel.replace("_", "")


BATCH_WORKLOAD = "batched512_2d_N32-512_markers100-20000_fourier_IB4"
SERVE_WORKLOAD = "serving_poisson2000_32sims_2d64-512_3d32-192_markers1e3-5e5_IB4_budget150GB"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--tune", action="store_true", help="run the autotuner on the helices workload")
    ap.add_argument("--no-tune", action="store_true", help="library defaults on the helices workload")
    ap.add_argument("--setting", default=None,
                    help="fixed plan setting k=v,... as printed under tuning.setting (helices or batched workload)")
    ap.add_argument("--kernel", default="IB_4", choices=sorted(KERNEL_WIDTHS),
                    help="delta kernel of the helices workload (the metric is quoted on IB_4)")
    ap.add_argument("--workload", default="all", choices=["all", "helices", "batched", "serving"],
                    help="all: the helices line (IB_4) with nested ib6, batched and serving results; "
                         "helices / batched / serving: that workload's line alone")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baselines (profiling runs)")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(value, world, device):
    """The largest value over the ranks (the job's time is its slowest
    rank's); a no-op for one rank."""
    if world <= 1:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def recorded_traffic():
    """profiles/traffic.json: {workload: {"setting": ..., "spread": bytes, ...}}."""
    try:
        with open(TRAFFIC) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.2)
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cuda_timer(stream):
    import torch

    def timed(fn, reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    return timed


# ---------------------------------------------------------------------------
# CPU baselines (the reference's per-patch CPU path, oracle port)
# ---------------------------------------------------------------------------
def make_markers():
    from ibamr_gb300 import workloads

    X = workloads.helices_and_uniform()
    rng = np.random.default_rng(workloads.SEED + 30)
    F = rng.standard_normal(X.size)
    return X, F


def helices_cpu(X, F, u_np, kernel, steps, warmup):
    """The reference's per-patch CPU flow on the whole helices workload: box
    patches cut by marker workload, four per host thread, worked through by
    every host thread; markers/s."""
    from oracle import ibx_oracle as oracle

    n = X.size // 3
    cores = os.cpu_count() or 1
    plan = oracle.CpuPlan(3, [N_GRID] * 3, kernel, X, threads=cores, boxes=4 * cores)
    f = np.zeros(3 * N_GRID ** 3)
    U = np.zeros(X.size)
    for _ in range(warmup):
        plan.step(F, f, u_np, U)
    t0 = time.perf_counter()
    for _ in range(steps):
        plan.step(F, f, u_np, U)
    dt = (time.perf_counter() - t0) / steps
    return {"value": n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "whole workload (%d markers, %d^3 grid) per step, %d box patches on %d threads, %d timed "
                      "steps" % (n, N_GRID, plan.patches, cores, steps), "ms_per_step": dt * 1e3}


def batched_problems():
    from ibamr_gb300 import workloads

    return [([N, N], X) for N, X in workloads.batched_2d(512)]


def batched_cpu(problems, F, steps=1, warmup=1):
    """The per-patch CPU path on every problem of the batch, one problem per
    task on a pool of host threads; markers/s."""
    import concurrent.futures

    from oracle import ibx_oracle as oracle

    moff = np.concatenate([[0], np.cumsum([X.size // 2 for _, X in problems])])
    cores = os.cpu_count() or 1
    work = []
    for k, (N, X) in enumerate(problems):
        vol = N[0] * N[1]
        Fk = np.ascontiguousarray(F[2 * moff[k]: 2 * moff[k + 1]])
        u = np.random.default_rng(100 + k).standard_normal(2 * vol)
        work.append((oracle.CpuPlan(2, N, "IB_4", X), Fk, np.zeros(2 * vol), u, np.zeros(X.size)))

    def run(w):
        plan, Fk, f, u, U = w
        plan.step(Fk, f, u, U)

    with concurrent.futures.ThreadPoolExecutor(max_workers=cores) as ex:
        for _ in range(warmup):
            list(ex.map(run, work))
        t0 = time.perf_counter()
        for _ in range(steps):
            list(ex.map(run, work))
        dt = (time.perf_counter() - t0) / steps
    m = int(moff[-1])
    return {"value": m / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "all %d problems (%d markers) per step, one problem per task on %d threads, %d timed steps"
                      % (len(problems), m, cores, steps), "ms_per_step": dt * 1e3}


def serving_specs(n_sims=32):
    from ibamr_gb300 import serving, workloads

    return [serving.SimSpec(sid, dim, N, X, F=F, u=u) for sid, dim, N, X, F, u in workloads.serving_mix(n_sims)]


def serving_cpu(specs):
    """The per-patch CPU path for one request of every simulation, one
    simulation per task on a pool of host threads; markers/s."""
    import concurrent.futures

    from oracle import ibx_oracle as oracle

    cores = os.cpu_count() or 1
    work = []
    for s in specs:
        vol = int(np.prod(s.N))
        work.append((oracle.CpuPlan(s.dim, s.N, "IB_4", s.X), np.ascontiguousarray(s.F, dtype=np.float64),
                     np.zeros(s.dim * vol), np.ascontiguousarray(s.u, dtype=np.float64).reshape(-1),
                     np.zeros(s.X.size)))

    def run(w):
        plan, F, f, u, U = w
        plan.step(F, f, u, U)

    with concurrent.futures.ThreadPoolExecutor(max_workers=cores) as ex:
        list(ex.map(run, work))
        t0 = time.perf_counter()
        list(ex.map(run, work))
        dt = time.perf_counter() - t0
    m = int(sum(s.n_markers for s in specs))
    return {"value": m / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "one request of each of the %d simulations (%d markers), one simulation per task on %d "
                      "threads" % (len(specs), m, cores), "ms_per_step": dt * 1e3}


# ---------------------------------------------------------------------------
# Reference arm: the CPU port of the reference's per-patch flow
# ---------------------------------------------------------------------------
def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    from ibamr_gb300 import workloads

    if args.workload == "batched":
        problems = batched_problems()
        nm = sum(X.size // 2 for _, X in problems)
        F = np.random.default_rng(workloads.SEED + 40).standard_normal(nm * 2)
        cpu = batched_cpu(problems, F, steps=args.steps, warmup=args.warmup)
        config = {"workload": BATCH_WORKLOAD, "kernel": "IB_4"}
    elif args.workload == "serving":
        cpu = serving_cpu(serving_specs())
        config = {"workload": SERVE_WORKLOAD, "kernel": "IB_4"}
    else:
        X, F = make_markers()
        u_np = np.random.default_rng(11).standard_normal(3 * N_GRID ** 3)
        cpu = helices_cpu(X, F, u_np, args.kernel, steps=args.steps, warmup=args.warmup)
        config = {"workload": helices_workload(args.kernel), "markers": X.size // 3, "grid": [N_GRID] * 3,
                  "kernel": args.kernel}
    line = {
        "impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": cpu["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": config,
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Helices workload (the headline configuration, and IB_6)
# ---------------------------------------------------------------------------
# FP64 rate of a GB300 (nominal, non-tensor), for the FP64 floor of a step
GB300_FP64_TFLOPS = 1.25


def fp64_fma_floor_ms(n_markers, dim, width):
    """Time the multiply-adds of one spread + interpolation in FP64 take at
    the GB300's nominal FP64 rate: dim components x width^dim stencil points
    per marker, one FMA each way -- a floor for any FP64 form of the step."""
    fmas = 2 * n_markers * dim * width ** dim
    return 2 * fmas / (GB300_FP64_TFLOPS * 1e12) * 1e3


def tile_index(X, N, edges):
    """Tile of each marker's cell (periodic unit box, N cells per side)."""
    P = np.asarray(X).reshape(-1, len(N))
    t = np.zeros(len(P), dtype=np.int64)
    stride = 1
    for d in range(len(N)):
        c = np.floor(P[:, d] * N[d]).astype(np.int64) % N[d]
        t += (c // edges[d]) * stride
        stride *= (N[d] + edges[d] - 1) // edges[d]
    return t


def pick_io_mode(plan, step_e2e, timed, steps, recapture=None):
    """Step mode of the end-to-end step (bin + spread + interpolate with
    their host transfers): the plan's own mode, the concurrent modes (with
    values going out the interpolation's stream comes first in modes 1 and
    4; both of one priority in mode 3), or mode 0 (interpolation first, its
    values' copy beside the spread), whichever measures fastest; leaves the
    plan (and the captured graph) in that mode."""
    best = None
    for m in dict.fromkeys([plan.step_mode, 1, 3, 4, 0]):
        plan.step_mode = m
        if recapture:
            recapture()
        for _ in range(2):
            step_e2e()
        t = timed(step_e2e, max(3, steps // 4))
        if best is None or t < best[1]:
            best = (m, t)
    plan.step_mode = best[0]
    if recapture:
        recapture()
    return best[0]


def helices_case(args, kernel, dev, world, setting_mode, with_cpu, steps, warmup):
    """One kernel on the 2M-marker workload: tuned or pinned plan, timed
    steps, phases, roofline, accuracy against the plain FP64 form, plain FP64
    rate, end to end with host buffers, CPU baseline."""
    import torch

    from ibamr_gb300 import ibx, tuning, workloads

    rank = dist_env()[0]
    W = KERNEL_WIDTHS[kernel]
    workload = helices_workload(kernel)
    X, F = make_markers()
    n = X.size // 3
    N = [N_GRID] * 3
    dx = [1.0 / N_GRID] * 3
    u_np = np.random.default_rng(11).standard_normal(3 * N_GRID ** 3)
    stream = torch.cuda.current_stream()
    timed = cuda_timer(stream)

    X_t = torch.tensor(X, device=dev)
    F_t = torch.tensor(F, dtype=torch.float32, device=dev)
    U_t = torch.zeros(3 * n, dtype=torch.float32, device=dev)
    f_t = [torch.zeros(N, dtype=torch.float32, device=dev) for _ in range(3)]
    u_t = [torch.tensor(u_np.reshape(3, *N)[a], dtype=torch.float32, device=dev) for a in range(3)]

    def prob(q, Xq, Q):
        return ibx.make_problem(3, ibx.SIDE, ibx.MODE_PERIODIC, [0] * 3, [N_GRID - 1] * 3, dx, [0.0] * 3, [1.0] * 3,
                                q, Xq, Q)

    def make_plan(shape):
        return ibx.Plan(prob(f_t, X_t, F_t), kernel, ibx.MIXED, interp_problems=[prob(u_t, X_t, U_t)],
                        tile_shape=shape)

    recorded = recorded_traffic().get(workload)
    tuned, source = None, "library defaults"
    if setting_mode == "tune":
        plan, tuned = tuning.autotune_shape(make_plan, reps=8)
        source = "autotuner"
    elif isinstance(setting_mode, str) and setting_mode not in ("defaults", "pinned"):
        fixed = tuning.parse_setting(setting_mode)
        plan = make_plan(fixed.get("tile_shape", 0))
        tuning.apply_setting(plan, fixed)
        source = "fixed"
    elif setting_mode == "pinned" and recorded and recorded.get("setting"):
        fixed = tuning.parse_setting(recorded["setting"])
        plan = make_plan(fixed.get("tile_shape", 0))
        tuning.apply_setting(plan, fixed)
        source = "autotuner's choice recorded with the ncu profile (profiles/traffic.json)"
    elif setting_mode == "pinned":
        plan, tuned = tuning.autotune_shape(make_plan, reps=8)
        source = "autotuner"
    else:
        plan = make_plan(0)
    setting = tuning.setting_string(tuning.setting_of(plan))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # One step (bin, then spread and interpolate concurrently) captured once
    # into a CUDA graph that keeps the plan's stream priorities
    # (ibx_plan_graph) and replayed, as a time stepper runs it; the kernels of
    # a replay are the ones counted at capture.
    for _ in range(warmup):
        plan.step()
    torch.cuda.synchronize()
    graph = plan.graph()
    per_step = graph.kernels
    for _ in range(warmup):
        graph.launch(stream)
    torch.cuda.synchronize()
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed_steps")  # profilers can select the timed launches by this range
    e0.record(stream)
    for _ in range(steps):
        graph.launch(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    launches = per_step * steps
    graph.close()
    barrier()
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1) / steps, world, dev)
    value = world * n / (ms * 1e-3)

    # per-phase timing (same stream) for the roofline
    reps = max(3, steps // 2)
    t_bin = timed(plan.bin, reps)
    t_spread = timed(plan.spread, reps)
    t_interp = timed(plan.interpolate, reps)
    T = workloads.touched_faces(X, 3, N, W)
    s_v = s_g = 4
    b_spread = n * 3 * (8 + s_v) + T * 2 * s_g
    b_interp = n * 3 * (8 + s_v) + T * s_g
    b_step = n * 3 * (8 + 2 * s_v) + T * 3 * s_g
    b_bin = n * 3 * 8  # binning reads the positions once
    peak, peak_kind = measured_peak()
    dom = max([("spread", t_spread, b_spread), ("interpolate", t_interp, b_interp), ("bin", t_bin, b_bin)],
              key=lambda z: z[1])
    traffic, traffic_note = None, "no ncu record for this setting"
    if recorded and recorded.get("setting") == setting:
        traffic = recorded.get(dom[0])
        traffic_note = "ncu DRAM bytes of the %s phase with this setting (profiles/traffic.json)" % dom[0]
    achieved = (dom[2] / (dom[1] * 1e-3)) / 1e9
    roofline = {"bound": "hbm", "kernel": dom[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_note,
                "peak_source": peak_kind,
                "step_achieved": (b_step / (ms * 1e-3)) / 1e9, "step_frac": (b_step / (ms * 1e-3)) / 1e9 / peak,
                "algorithmic_bytes": {"spread": b_spread, "interpolate": b_interp, "bin": b_bin, "step": b_step,
                                      "touched_faces": T}}

    # accuracy of the mixed form against the plain FP64 form
    f_t2 = [torch.zeros(N, dtype=torch.float32, device=dev) for _ in range(3)]
    plan_e = ibx.Plan(prob(f_t2, X_t, F_t), kernel, ibx.MIXED, tile_shape=plan.tile_shape[0])
    plan_e.set_tuning(*plan.tuning())
    plan_e.visit_kernel = plan.visit_kernel
    plan_e.unit_cap = plan.unit_cap
    plan_e.bin()
    plan_e.spread()
    fd = [torch.zeros(N, dtype=torch.float64, device=dev) for _ in range(3)]
    ud = [t.double() for t in u_t]
    Fd = torch.tensor(F, device=dev)
    Ud = torch.zeros(3 * n, dtype=torch.float64, device=dev)
    ibx.spread(prob(fd, X_t, Fd), kernel, ibx.FP64)
    ibx.interpolate(prob(ud, X_t, Ud), kernel, ibx.FP64)
    torch.cuda.synchronize()
    err_f = max(float((f_t2[a].double() - fd[a]).abs().max()) for a in range(3)) / max(
        float(fd[a].abs().max()) for a in range(3))
    plan.interpolate()
    torch.cuda.synchronize()
    err_U = float((U_t.double() - Ud).abs().max() / Ud.abs().max())
    plan_e.close()
    del f_t2

    # plain FP64 form (marker-parallel, FP64 atomics) on the same workload
    def step_plain():
        ibx.spread(prob(fd, X_t, Fd), kernel, ibx.FP64)
        ibx.interpolate(prob(ud, X_t, Ud), kernel, ibx.FP64)

    step_plain()
    ms_plain = timed(step_plain, max(2, steps // 5))
    # the same form over the markers sorted into tile order once, outside the
    # timed region (the locality a binning gives the marker-parallel form)
    order = np.argsort(tile_index(X, [N[0]] * 3, plan.tile_shape[1]), kind="stable")
    X_s = torch.tensor(X.reshape(-1, 3)[order].reshape(-1), device=dev)
    F_s = torch.tensor(F.reshape(-1, 3)[order].reshape(-1), device=dev)

    def step_plain_sorted():
        ibx.spread(prob(fd, X_s, F_s), kernel, ibx.FP64)
        ibx.interpolate(prob(ud, X_s, Ud), kernel, ibx.FP64)

    step_plain_sorted()
    ms_plain_sorted = timed(step_plain_sorted, max(2, steps // 5))
    del fd, ud, Fd, Ud, X_s, F_s

    # end to end through the C ABI with host buffers (ibx_plan_step_io): the
    # positions go up first, the forces behind them beside the binning (which
    # needs only the positions), spread and interpolation run on two streams,
    # the velocities come down as soon as the interpolation ends; each step
    # starts after the previous one has delivered its velocities
    Xh = torch.tensor(X).pin_memory()
    Fh = torch.tensor(F, dtype=torch.float32).pin_memory()
    Uh = torch.empty(3 * n, dtype=torch.float32).pin_memory()
    io = dict(in_X=[(X_t, Xh)], in_Q=[(F_t, Fh)], out_Q=[(Uh, U_t)])
    io_graph = [None]

    def recapture():
        if io_graph[0] is not None:
            io_graph[0].close()
        io_graph[0] = None
        plan.step_io(**io)
        torch.cuda.synchronize()
        io_graph[0] = plan.graph(**io)

    def step_e2e():
        io_graph[0].launch(stream)

    # the step mode of the transfer step (one CUDA graph holding the
    # transfers): the tuned one, or the interpolation first with the
    # velocities' copy beside the spread, whichever is faster
    io_mode = pick_io_mode(plan, step_e2e, timed, steps, recapture=recapture)

    for _ in range(2):
        step_e2e()
    barrier()
    ms_e2e = max_over_ranks(timed(step_e2e, steps), world, dev)
    e2e = {"value": world * n / (ms_e2e * 1e-3), "unit": UNIT, "h2d_bytes_per_step": X.size * 8 + F.size * 4,
           "d2h_bytes_per_step": 3 * n * 4, "ms_per_step": ms_e2e, "call": "ibx_plan_step_io (in the graph)",
           "step_mode": io_mode}
    io_graph[0].close()
    io_graph[0] = None
    status = plan.status()
    tile_edges = list(plan.tile_shape[1])
    plan.close()
    del f_t, u_t, X_t, F_t, U_t
    torch.cuda.empty_cache()
    cpu = None
    if with_cpu and rank == 0:
        cpu = helices_cpu(X, F, u_np, kernel, steps=2 if kernel == "IB_4" else 1, warmup=1)
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE, "data": "synthetic (seeded)",
        "config": {"workload": workload, "markers": n, "grid": N, "kernel": kernel, "centering": "side",
                   "precision": "mixed", "launch": "one CUDA graph per step",
                   "l2": "inputs larger than L2 (2 x 201 MB grids, 72 MB markers)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "phases_ms": {"bin": t_bin, "spread": t_spread, "interpolate": t_interp},
        "plain_fp64": {"value": world * n / (ms_plain * 1e-3), "ms_per_step": ms_plain,
                       "tile_order_ms_per_step": ms_plain_sorted,
                       "fp64_fma_floor_ms": fp64_fma_floor_ms(n, 3, KERNEL_WIDTHS[kernel])},
        "mixed_vs_plain": ms_plain / ms,
        "error_vs_fp64": {"spread": err_f, "interpolate": err_U, "tolerance": 1e-5},
        "status": ibx.status_string(status),
        "tuning": {
            "setting": setting, "tile_edges": tile_edges, "source": source,
            "tuned_step_ms": None if tuned is None else tuned["ms"],
            "per_shape": None if tuned is None else {
                str(k): [list(v[0]), round(v[1], 4)] for k, v in tuned["per_shape"].items()}},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "clocks": clocks,
    }


# ---------------------------------------------------------------------------
# Batched workload: 512 independent 2D periodic problems, one CUDA graph
# ---------------------------------------------------------------------------
def batched_case(args, dev, world, with_cpu, steps, warmup, setting=None):
    import torch

    from ibamr_gb300 import batch, ibx, tuning, workloads

    rank = dist_env()[0]
    problems = batched_problems()
    B = batch.BatchedProblems(problems, dim=2, kernel="IB_4", device=dev, tune=False)
    nm = int(B.marker_offsets[-1])
    F = np.random.default_rng(workloads.SEED + 40).standard_normal(nm * 2)
    B.F.copy_(torch.tensor(F, dtype=torch.float32))
    gen = torch.Generator(device=dev)
    gen.manual_seed(workloads.SEED + 41)
    B.u.copy_(torch.randn(B.u.numel(), generator=gen, device=dev))
    if setting:
        B.configure(tuning.parse_setting(setting))
    else:
        B.autotune(reps=8)  # on the batch's own forces and velocities
    setting = tuning.setting_string(tuning.setting_of(B.plan))
    stream = torch.cuda.current_stream()
    timed = cuda_timer(stream)

    l0 = ibx.kernel_launches()
    B.step()
    per_step = ibx.kernel_launches() - l0
    B.capture()
    for _ in range(warmup):
        B.replay()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.nvtx.range_push("timed_steps")
    ms = timed(B.replay, steps)
    torch.cuda.nvtx.range_pop()
    clocks = sampler.stop()
    ms = max_over_ranks(ms, world, dev)
    value = world * nm / (ms * 1e-3)

    reps = max(3, steps // 2)
    t_bin = timed(B.plan.bin, reps)
    t_spread = timed(B.plan.spread, reps)
    t_interp = timed(B.plan.interpolate, reps)
    T = sum(workloads.touched_faces(X, 2, N, 4) for N, X in problems)
    b_spread = nm * 2 * (8 + 4) + T * 2 * 4
    b_interp = nm * 2 * (8 + 4) + T * 4
    b_step = nm * 2 * (8 + 8) + T * 3 * 4
    b_bin = nm * 2 * 8
    peak, peak_kind = measured_peak()
    dom = max([("spread", t_spread, b_spread), ("interpolate", t_interp, b_interp), ("bin", t_bin, b_bin)],
              key=lambda z: z[1])
    achieved = (dom[2] / (dom[1] * 1e-3)) / 1e9
    roofline = {"bound": "hbm", "kernel": dom[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                "step_achieved": (b_step / (ms * 1e-3)) / 1e9, "step_frac": (b_step / (ms * 1e-3)) / 1e9 / peak,
                "algorithmic_bytes": {"spread": b_spread, "interpolate": b_interp, "bin": b_bin, "step": b_step,
                                      "touched_faces": T}}

    # accuracy against the plain FP64 form (all 512 problems in one call each)
    f64 = [[torch.zeros(N[::-1], dtype=torch.float64, device=dev) for _ in range(2)] for N, _ in problems]
    u64 = [[t.double() for t in B.grid("u", k)] for k in range(len(problems))]
    F64 = torch.tensor(F, device=dev)
    U64 = torch.zeros(nm * 2, dtype=torch.float64, device=dev)
    sp, ip = [], []
    for k, (N, X) in enumerate(problems):
        a, b = int(B.marker_offsets[k]) * 2, int(B.marker_offsets[k + 1]) * 2
        mk = lambda q, Q: ibx.make_problem(2, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [N[0] - 1, N[1] - 1],
                                           [1.0 / N[0], 1.0 / N[1]], [0.0, 0.0], [1.0, 1.0], q, B.X[a:b], Q[a:b])
        sp.append(mk(f64[k], F64))
        ip.append(mk(u64[k], U64))

    def step_plain():
        ibx.spread(sp, "IB_4", ibx.FP64)
        ibx.interpolate(ip, "IB_4", ibx.FP64)

    B.f.zero_()
    B.step()
    step_plain()
    torch.cuda.synchronize()
    err_f = max(float((B.grid("f", k)[a].double() - f64[k][a]).abs().max()) for k in range(len(problems))
                for a in range(2)) / max(float(f64[k][a].abs().max()) for k in range(len(problems)) for a in range(2))
    err_U = float((B.U.double() - U64).abs().max() / U64.abs().max())
    ms_plain = timed(step_plain, max(2, steps // 5))
    del f64, u64, sp, ip, F64, U64

    # end to end: positions and forces in from pinned host memory, velocities out
    Xh = B.X.cpu().pin_memory()
    Fh = B.F.cpu().pin_memory()
    Uh = torch.empty(nm * 2, dtype=torch.float32).pin_memory()

    # one CUDA graph per step holding the transfers (ibx_plan_step_io):
    # positions up, forces up beside the binning, velocities down beside the
    # spread
    io = B.host_io(Xh, Fh, Uh)
    B.capture(io)

    def step_e2e():
        B.replay()

    io_mode = pick_io_mode(B.plan, step_e2e, timed, steps, recapture=lambda: B.capture(io))
    step_e2e()
    ms_e2e = max_over_ranks(timed(step_e2e, steps), world, dev)
    e2e = {"value": world * nm / (ms_e2e * 1e-3), "unit": UNIT, "h2d_bytes_per_step": nm * 2 * (8 + 4),
           "d2h_bytes_per_step": nm * 2 * 4, "ms_per_step": ms_e2e, "call": "ibx_plan_step_io (in the graph)",
           "step_mode": io_mode}
    tuned = B.tuning
    status = B.status()
    B.close()
    torch.cuda.empty_cache()
    cpu = batched_cpu(problems, F) if with_cpu and rank == 0 else None
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE,
        "data": "synthetic (seeded)",
        "config": {"workload": BATCH_WORKLOAD, "problems": len(problems), "markers": nm,
                   "grid_values": int(sum(2 * N[0] * N[1] for N, _ in problems)), "kernel": "IB_4",
                   "centering": "side", "precision": "mixed", "launch": "one CUDA graph per step",
                   "l2": "inputs larger than L2 (2 x 286 MB grids)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "phases_ms": {"bin": t_bin, "spread": t_spread, "interpolate": t_interp},
        "plain_fp64": {"value": world * nm / (ms_plain * 1e-3), "ms_per_step": ms_plain},
        "mixed_vs_plain": ms_plain / ms,
        "error_vs_fp64": {"spread": err_f, "interpolate": err_U, "tolerance": 1e-5},
        "status": ibx.status_string(status),
        "tuning": {
            "setting": setting, "source": "autotuner" if tuned is not None else "fixed",
            "tuned_step_ms": None if tuned is None else tuned["ms"],
            "per_shape": None if tuned is None else {
                str(k): [list(v[0]), round(v[1], 4)] for k, v in tuned["per_shape"].items()}},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": per_step * steps,
        "kernels_per_step": per_step, "clocks": clocks,
    }


# ---------------------------------------------------------------------------
# Serving workload: Poisson request stream over resident simulations
# ---------------------------------------------------------------------------
def serving_case(args, dev, world, with_cpu, steps):
    import torch

    from ibamr_gb300 import serving, workloads

    rank = dist_env()[0]
    specs = serving_specs()
    backend = serving.CudaBackend("IB_4", device=dev)
    srv = serving.Server(backend, 150 * 10 ** 9, n_slots=8)
    for s in specs:
        srv.register(s)
    n_req = max(2000, 200 * steps)
    warm = serving.poisson_requests(2000.0, 2 * len(specs), [s.sid for s in specs], seed=1)
    warm = [serving.Request(i, 0.0, specs[i % len(specs)].sid) for i in range(len(specs))] + warm
    warm = [serving.Request(i, r.arrival, r.sid) for i, r in enumerate(warm)]
    srv.run(warm)  # every simulation resident, kernels loaded
    torch.cuda.synchronize()
    reqs = serving.poisson_requests(2000.0, n_req, [s.sid for s in specs], seed=2)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    l0 = backend.kernel_launches  # graph replays count the kernels of the captured step
    out = srv.run(reqs)
    torch.cuda.synchronize()
    launches = backend.kernel_launches - l0
    # capacity: the same number of requests all queued at once
    burst = [serving.Request(r.rid, 0.0, r.sid) for r in reqs[: max(1000, n_req // 2)]]
    sat = srv.run(burst)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    srv.close()
    torch.cuda.empty_cache()
    # algorithmic bytes of one request of each simulation (markers and
    # touched faces), summed over the saturated run's requests
    b_sim = {s.sid: s.n_markers * s.dim * (8 + 8) + 3 * 4 * workloads.touched_faces(s.X, s.dim, s.N, 4)
             for s in specs}
    span = len(burst) / sat["requests_per_s"]
    achieved = sum(b_sim[r.sid] for r in burst) / span / 1e9
    peak, peak_kind = measured_peak()
    cpu = serving_cpu(specs) if with_cpu and rank == 0 else None
    value = world * out["markers_per_s"]
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": n_req,
        "warmup": len(warm), "ms_per_step": out["mean_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE, "data": "synthetic (seeded)",
        "config": {"workload": SERVE_WORKLOAD, "simulations": len(specs), "requests": n_req,
                   "arrival_rate_per_s": 2000.0, "slots": 8, "budget_bytes": 150 * 10 ** 9,
                   "markers_per_simulation": "log-uniform in [1e3, 5e5]", "kernel": "IB_4",
                   "parallelism": "replicas" if world > 1 else "single"},
        "latency_ms": {"p50": out["p50_ms"], "p99": out["p99_ms"], "mean": out["mean_ms"]},
        "requests_per_s": out["requests_per_s"], "max_queue": out["max_queue"],
        "resident_bytes": out["used_bytes"], "evictions": out["evictions"],
        "saturated": {"requests": len(burst), "markers_per_s": sat["markers_per_s"],
                      "requests_per_s": sat["requests_per_s"], "p50_ms": sat["p50_ms"], "p99_ms": sat["p99_ms"]},
        "roofline": {"bound": "hbm", "kernel": "whole request (saturated run)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_source": peak_kind},
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "request loop through the public API; simulation state resident on the device"},
        "gpu_launches": launches, "clocks": clocks,
    }


NESTED_KEYS = ("value", "unit", "ms_per_step", "steps", "warmup", "config", "phases_ms", "plain_fp64",
               "mixed_vs_plain", "error_vs_fp64", "status", "tuning", "roofline", "e2e", "cpu_baseline",
               "gpu_launches", "kernels_per_step", "latency_ms", "requests_per_s", "saturated", "clocks",
               "max_queue", "resident_bytes", "evictions")


def nested(line):
    return {k: line[k] for k in NESTED_KEYS if k in line}


def fortran_abi_case(dev, reps=7):
    """The reference's own entry points, called as LEInteractor calls them:
    lagrangian_ib_4_spread3d_ and lagrangian_ib_4_interp3d_ (the Fortran ABI
    of libibx) on one ghosted 128^3 cell patch of depth 3 with 200,000
    markers, every array a host array (staged through the library's pool,
    copied in and back per call), against the same calls with device
    arrays.  One step = one spread + one interpolation; the median of the
    separately timed calls."""
    import ctypes

    import numpy as np
    import torch

    from ibamr_gb300 import ibx

    L = ibx.lib()
    n, N, g, depth = 200_000, 128, 3, 3
    rng = np.random.default_rng(5)
    X = rng.uniform(0.0, 1.0, (n, 3)).reshape(-1)
    V = rng.standard_normal(n * depth)
    u = np.zeros(depth * (N + 2 * g) ** 3)
    idx = np.arange(n, dtype=np.int32)
    sh = np.zeros(3 * n)
    dx = np.full(3, 1.0 / N)
    xl, xu = np.zeros(3), np.ones(3)
    ri = lambda v: ctypes.byref(ctypes.c_int(int(v)))
    box = [ri(0), ri(N - 1)] * 3
    gw = [ri(g)] * 3

    def pt(a):
        return ctypes.c_void_p(a.data_ptr()) if isinstance(a, torch.Tensor) else a.ctypes.data_as(ctypes.c_void_p)

    def step(arrs):
        uu, XX, VV, ii, ss = arrs
        L.lagrangian_ib_4_spread3d_(pt(dx), pt(xl), pt(xu), ri(depth), pt(ii), pt(ss), ri(n), pt(XX), pt(VV),
                                    *box, *gw, pt(uu))
        L.lagrangian_ib_4_interp3d_(pt(dx), pt(xl), pt(xu), ri(depth), *box, *gw, pt(uu), pt(ii), pt(ss), ri(n),
                                    pt(XX), pt(VV))

    def wall(arrs):
        # the median of separately timed calls: one call disturbed by
        # something else on the machine does not move it
        step(arrs)
        torch.cuda.synchronize()
        times = []
        for _ in range(reps):
            t0 = time.perf_counter()
            step(arrs)
            torch.cuda.synchronize()
            times.append((time.perf_counter() - t0) * 1e3)
        return float(np.median(times))

    host = (u, X, V.copy(), idx, sh)
    devs = tuple(torch.tensor(a, device=dev) for a in host)
    ms_h = wall(host)
    ms_d = wall(devs)
    return {"call": "lagrangian_ib_4_spread3d_ + lagrangian_ib_4_interp3d_", "markers": n,
            "patch": "128^3 cells, ghost width 3, depth 3, FP64", "host_arrays_ms": ms_h, "device_arrays_ms": ms_d,
            "host_arrays_markers_per_s": n / (ms_h * 1e-3), "device_arrays_markers_per_s": n / (ms_d * 1e-3),
            # spread: u in and out, X, V, indices, shifts in; interpolation: u, X, V, indices, shifts in, V out
            "host_bytes_per_step": int(8 * (3 * u.size + 2 * X.size + 3 * V.size + 2 * sh.size) + 4 * 2 * idx.size)}


def run_ours(args):
    import torch

    from ibamr_gb300 import ibx

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    ibx.lib()
    with_cpu = not args.no_cpu
    if args.setting:
        mode = args.setting
    elif args.tune:
        mode = "tune"
    elif args.no_tune:
        mode = "defaults"
    else:
        mode = "pinned"
    if args.workload == "batched":
        line = batched_case(args, dev, world, with_cpu, args.steps, args.warmup, setting=args.setting)
    elif args.workload == "serving":
        line = serving_case(args, dev, world, with_cpu, args.steps)
    else:
        line = helices_case(args, args.kernel, dev, world, mode, with_cpu, args.steps, args.warmup)
        if args.workload == "all":
            line["ib6"] = nested(helices_case(args, "IB_6", dev, world, "tune", with_cpu, args.steps,
                                              args.warmup))
            line["batched"] = nested(batched_case(args, dev, world, with_cpu, args.steps, args.warmup))
            line["serving"] = nested(serving_case(args, dev, world, with_cpu, args.steps))
            line["fortran_abi"] = fortran_abi_case(dev)
            # the other kernels of the path on the same workload (autotuned, no CPU baseline)
            line["kernels"] = {k: {key: v for key, v in helices_case(args, k, dev, world, "tune", False, args.steps,
                                                                     args.warmup).items()
                                   if key in ("value", "unit", "ms_per_step", "phases_ms", "mixed_vs_plain",
                                              "error_vs_fp64", "roofline", "e2e", "status")}
                               for k in ("IB_3", "PIECEWISE_CUBIC", "BSPLINE_4")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse_args()
    if args.kernel != "IB_4" and args.workload not in ("helices", "all"):
        raise SystemExit("--kernel applies to the helices workload")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
