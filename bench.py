"""Benchmark of the immersed-boundary step on GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--workload spheres3d_256|spheres3d_384|cylinder2d|cylinder2d_slip]
                [--precision fp64|mixed]
                [--sweep-form auto|split|fused]

One step = one time step of the whole case (snapshot, predictor, RHS,
iter_max red-black SOR iterations, projection, boundary).  Default workload:
the 3D drop-in case -- unit cube on a 256^3 grid, 32 seeded spheres, plain
FP64, iter_max=100, omega=1.7 -- with synthetic (seeded) porosity.

Prints one JSON line.  `value` is device time (CUDA events on the case's
stream) with the fields resident in HBM; `e2e` is the same metric through the
C ABI with pinned host buffers copied in and out every step: pf_step_host
(one step from host fields to host fields, the input copies overlapped with
the predictor), and under `three_calls` the same through pf_set_state +
pf_step + pf_get_state.  With --gpus N > 1 (torchrun) every rank advances
its own replica of the case (no exchange between ranks: the path shards by
case), and `value` is the sum over ranks over the max-over-ranks time.

--impl reference times the CPU restatement of the reference's OpenMP step
(the oracle; the reference is Fortran and no Fortran compiler is available)
on all host cores for the same workload and metric.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s at max|div u|<1e-6 (batched FP32+FP64-DC vs plain FP64); p50/p99"
UNIT = "Mcell-steps/s"


def workload(name: str, precision: str):
    from pixelflow_gb300 import geometry as G
    if name in ("spheres3d_256", "spheres3d_384", "spheres3d_192", "spheres3d_128", "spheres3d_64"):
        nn = int(name.split("_")[1])
        s = G.settings_spheres_3d(precision=precision)
        shape = (nn, nn, nn)
        vals = G.spheres_3d(nn, nn, nn)
        desc = dict(workload=f"3D ibm3 unit cube {nn}^3, 32 seeded spheres (seed 0), tanh edge 2 cells",
                    grid=list(shape), nu=s.xnue, dt=s.time / s.istep_max, iter_max=s.iter_max,
                    omega=s.relux_factor)
    elif name in ("cylinder2d", "cylinder2d_slip"):
        slip = name.endswith("_slip")
        s = G.settings_cylinder_2d(precision=precision, slip_y=slip)
        shape = (512, 256)
        vals = G.cylinder_2d()
        desc = dict(workload="2D ibm2 cylinder 512x256, D=0.1 at (0.5,0.5), Re=100"
                    + (", symmetry (slip) rows top and bottom" if slip else ", periodic y"), grid=list(shape),
                    nu=s.xnue, dt=s.time / s.istep_max, iter_max=s.iter_max, omega=s.relux_factor)
    else:
        raise SystemExit(f"unknown workload {name}")
    if precision == "mixed":
        desc.update(outer_passes=s.outer_max, inner_sweeps=s.inner_sweeps)
    desc["precision"] = precision
    return s, shape, vals, desc


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def fp64_peak_tflops(n: int = 4096, reps: int = 5) -> float:
    """FP64 arithmetic peak of this GPU as delivered by cuBLAS DGEMM (2 n^3
    flops, best of `reps`, CUDA events): the roof of the FP64 kernels."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best / 1e12


def ncu_traffic(name: str):
    """Per-launch DRAM bytes of the dominant kernel from a committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(name)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def stage_roofline(stage_ms, steps, cells, dim, s, precision, peak, peak_kind):
    """HBM roofline of every stage of the step: device time per step (CUDA
    events between the stages), the stage's algorithmic bytes per step
    (words per cell: predictor 7 (2D 5), RHS 5 (4), SOR 5 per iteration,
    projection + boundary 7 (5); FP64 words of 8 B, and in the precision
    form FP32 words of 4 B for the predictor's stencils and the sweeps), and
    the achieved fraction of the measured HBM copy peak."""
    sweeps = s.iter_max if precision == "fp64" else s.outer_max * s.inner_sweeps
    w8, w4 = 8, (8 if precision == "fp64" else 4)
    words = {"predictor": ((7 if dim == 3 else 5), w4), "rhs": ((5 if dim == 3 else 4), w8),
             "sor": (5 * sweeps, w4), "projection_boundary": ((7 if dim == 3 else 5), w8)}
    out = {}
    for k, ms in stage_ms.items():
        per_step = ms / max(steps, 1)
        nw, wsz = words[k]
        alg = cells * nw * wsz
        gbs = alg / (per_step / 1e3) / 1e9 if per_step > 0 else 0.0
        out[k] = {"ms_per_step": per_step, "alg_bytes_per_step": alg, "achieved_gbs": gbs,
                  "frac": gbs / peak if peak else None}
    out["peak_gbs"] = peak
    out["peak_source"] = peak_kind
    return out


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(settings, shape, vals, budget_s: float = 20.0, max_steps: int = 5):
    """The oracle (OpenMP, all host threads) on a bounded sample of the workload."""
    from oracle.oracle import OracleCase
    c = OracleCase(settings, shape, vals)
    c.initialize()
    cells = int(np.prod(shape))
    times = []
    while len(times) < max_steps and sum(times) < budget_s:
        t0 = time.perf_counter()
        c.step(1)
        times.append(time.perf_counter() - t0)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": cells * len(times) / sum(times) / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{len(times)} full steps of the same case from the initial state "
                      f"({sum(times):.1f} s, oracle = C restatement of the reference OpenMP step, FP64)"}


def _plain_sequential(items, steps: int):
    """The plain FP64 single-case step on every given case, one case after
    another: each case is created, stepped once (its step graph captured),
    then `steps` graph replays are timed on the host clock (launches
    included).  items: (settings, shape, porosity values or None, shapes)."""
    from pixelflow_gb300.solver import Case
    tot_cells, tot_s = 0, 0.0
    for s, shape, vals, shapes in items:
        s = s.replace(precision="fp64")
        c = Case(s, shape, vals) if vals is not None else Case.from_shapes(s, shape, shapes)
        with c:
            c.initial_conditions()
            c.step(1)
            c.synchronize()
            t0 = time.perf_counter()
            c.step(steps)
            c.synchronize()
            tot_s += time.perf_counter() - t0
        tot_cells += int(np.prod(shape)) * steps
    return {"value": tot_cells / tot_s / 1e6, "unit": UNIT, "cases": len(items), "steps_each": steps,
            "timing": "host clock around graph replays, one case after another"}


def bench_batch(ncases: int = 512, steps: int = 20, warmup_steps: int = 2, seed: int = 0,
                baseline_steps: int = 20, large_cells: int = 100000, plain_value: float = 0.0,
                schedule_bound: float = 1e-6):
    """The batched form: `ncases` independent 2D cases of uneven size (nx, ny in
    {64, 96, ..., 512}, 1-4 circles/ellipses, Re 50-400 capped at cell
    Reynolds number 2, dt at CFL 0.2 of the predictor's stability limit,
    porosity threshold 0.1), precision form (FP32 sweeps in FP64 defect
    correction, the schedule from the autotuner), advanced by the
    persistent batch kernel.  Reports
    device-timed aggregate Mcell-steps/s over the cases that stay finite and,
    as the comparison, the plain FP64 single-case step run on every case, one
    after another."""
    from pixelflow_gb300 import geometry as G
    from pixelflow_gb300.autotune import tune_batch, tune_batch_schedule
    from pixelflow_gb300.batch import Batch
    cases = G.batch_cases_2d(ncases, seed=seed)
    sched, sched_trials = tune_batch_schedule(cases, bound=schedule_bound, use_cache=False)
    t0 = time.perf_counter()
    b = Batch(max_cases=ncases, large_cells=large_cells)
    slots = [b.add(c.settings.replace(outer_max=sched[0], inner_sweeps=sched[1]), (c.m, c.n), c.porosity())
             for c in cases]
    setup_s = time.perf_counter() - t0
    best, trials = tune_batch(b, slots, steps=warmup_steps, use_cache=False)
    l0 = b.kernel_launches()
    b.step_slots(slots, [steps] * len(slots))
    ms = b.last_ms()
    launches = b.kernel_launches() - l0
    mem = b.memory()[0]
    graph_stats = dict(zip(("captured", "replays"), b.graph_stats()))
    finite = [bool(np.isfinite(b.norms(sl)[0])) for sl in slots]
    b.close()
    cells = sum(c.m * c.n for c, ok in zip(cases, finite) if ok)
    value = cells * steps / (ms / 1e3) / 1e6
    plain = _plain_sequential([(c.settings, (c.m, c.n), c.porosity(), None) for c in cases], baseline_steps)
    out = {"workload": f"{ncases} 2D ibm2 cases, nx,ny in 64..512 step 32, seed {seed}, mixed "
                       f"{sched[0]}x{sched[1]} (autotuned within {schedule_bound:g} relative L2 of FP64), "
                       f"cases > {large_cells} cells as full-GPU step graphs beside the persistent kernel",
           "cells": cells, "value": value, "unit": UNIT, "steps": steps, "ms": ms,
           "value_counts": "cell-steps of the cases finite after the timed steps",
           "launches_in_timed_region": launches, "setup_s": setup_s, "device_bytes": mem,
           "nonfinite_cases_after_timed_steps": len(finite) - sum(finite),
           "autotune": {"best": list(best), "trials": trials, "schedule": list(sched),
                        "schedule_bound": schedule_bound, "schedule_trials": sched_trials},
           "graph_stats": graph_stats,
           "plain_fp64_sequential": plain,
           "speedup_vs_plain_fp64_sequential": value / plain["value"]}
    if plain_value:
        out["speedup_vs_plain_fp64_256"] = value / plain_value
    return out


def bench_serving(count: int = 32, rate: float = 200.0, seed: int = 0, chunk: int = 25,
                  baseline_steps: int = 20, large_cells: int = 100000, policy: str = "srpt_fill",
                  plain_value: float = 0.0, schedule_bound: float = 0.0):
    """The serving form: `count` requests with Poisson arrivals (mean `rate`
    per second), 70 % 2D (128^2-1024^2) / 30 % 3D (64^3-192^3, 4-16 spheres),
    100-1000 steps each, admitted by a 150 GB HBM budget into one resident
    batch: cases up to `large_cells` cells in the persistent launch, larger
    ones as full-GPU step graphs on their own streams beside it.  Latency is
    wall-clock from arrival to the result (fields and norms) on the host.
    baseline_steps > 0 adds the plain FP64 step run on every request, one
    after another, for that many steps each."""
    from pixelflow_gb300 import geometry as G
    from pixelflow_gb300.serve import Server, summarize
    reqs = G.serving_requests(count=count, rate=rate, seed=seed)
    with Server(chunk=chunk, cluster=8, threads=512, keep_state=False, large_cells=large_cells,
                policy=policy) as srv:
        tuned, tune_s = None, 0.0
        if schedule_bound > 0:
            # the autotuner's schedule per 3D size (set-up, before the stream starts)
            tt = time.perf_counter()
            tuned = srv.tune_schedules(reqs, schedule_bound)
            tune_s = time.perf_counter() - tt
        t0 = time.perf_counter()
        res = srv.run(reqs, realtime=True)
        wall = time.perf_counter() - t0
        summ = summarize(res, wall)
        summ.update(rounds=srv.rounds, device_ms=srv.device_ms, peak_device_bytes=srv.peak_bytes, policy=policy,
                    max_waiting=srv.max_waiting)
        if tuned is not None:
            summ["schedules"] = {"bound": schedule_bound, "tune_s": tune_s, "by_size": tuned,
                                 "other_sizes": "4 x 25"}
    summ["workload"] = (f"{count} requests, Poisson {rate:g}/s, 70% 2D 128^2-1024^2 / 30% 3D 64^3-192^3, "
                        f"100-1000 steps, 150 GB budget, chunk {chunk}, large cases > {large_cells} cells "
                        f"on own streams, round policy {policy}")
    if baseline_steps:
        plain = _plain_sequential([(r.settings, r.shape, None, r.shapes) for r in reqs], baseline_steps)
        summ["plain_fp64_sequential"] = plain
        summ["speedup_vs_plain_fp64_sequential"] = summ["mcell_steps_per_s"] / plain["value"]
    if plain_value:
        summ["speedup_vs_plain_fp64_256"] = summ["mcell_steps_per_s"] / plain_value
    return summ


def bench_serving_rates(rates=(0.5, 1.0, 2.0), count: int = 32, seed: int = 0, schedule_bound: float = 0.0):
    """The serving form at sustainable arrival rates: per rate, `count`
    requests of the same mix; p50/p99 latency, the aggregate, the longest
    queue, and the latency growth (mean latency of the last quarter of the
    arrivals over the first quarter: about 1 while the queue stays bounded,
    growing with the backlog beyond the GPU's capacity)."""
    out = []
    for r in rates:
        from pixelflow_gb300 import geometry as G
        from pixelflow_gb300.serve import Server, summarize
        reqs = G.serving_requests(count=count, rate=r, seed=seed)
        with Server(chunk=25, cluster=8, threads=512, keep_state=False, policy="srpt_fill") as srv:
            if schedule_bound > 0:
                srv.tune_schedules(reqs, schedule_bound)  # cached from the first tuning
            t0 = time.perf_counter()
            res = srv.run(reqs, realtime=True)
            wall = time.perf_counter() - t0
            summ = summarize(res, wall)
            summ["max_waiting"] = srv.max_waiting
        lat = [x.latency_s for x in sorted(res, key=lambda x: x.arrival_s)]
        q = max(1, len(lat) // 4)
        summ["latency_growth"] = float(np.mean(lat[-q:]) / max(np.mean(lat[:q]), 1e-9))
        summ["rate_per_s"] = r
        summ["offered_mcell_steps_per_s"] = sum(x.cells * x.steps for x in reqs) / max(reqs[-1].arrival_s, 1e-9) / 1e6
        out.append(summ)
    bounded = [x["rate_per_s"] for x in out if x["latency_growth"] < 2.0 and x["max_waiting"] <= 2]
    return {"workload": f"{count} requests per rate, the serving mix, round policy srpt_fill",
            "rates": out, "bounded_up_to_per_s": max(bounded) if bounded else None,
            "bounded_rule": "latency growth < 2 and at most 2 requests waiting for admission"}


def run_reference(args):
    rank, world, _ = dist_setup()
    if rank != 0:
        barrier(world)
        return
    s, shape, vals, desc = workload(args.workload, "fp64")
    # the same workload keys as the GPU arm's line
    desc.update(parallelism=f"replicas{world}" if world > 1 else "single",
                l2="working set > 129 MB L2 (no flush needed)")
    from oracle.oracle import OracleCase
    cells = int(np.prod(shape))
    c = OracleCase(s, shape, vals)
    c.initialize()
    for _ in range(min(args.warmup, 1)):
        c.step(1)
    budget = float(os.environ.get("PF_REFERENCE_BUDGET_S", "150"))
    times = []
    while len(times) < args.steps and sum(times) < budget:
        t0 = time.perf_counter()
        c.step(1)
        times.append(time.perf_counter() - t0)
    value = cells * len(times) / sum(times) / 1e6
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    sample = (f"{len(times)} of {args.steps} requested steps timed (cap {budget:.0f} s), "
              f"{min(args.warmup, 1)} warm-up; oracle = C restatement of the reference OpenMP step")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": len(times),
           "warmup": min(args.warmup, 1), "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": desc,
           "latency_ms": {"p50": 1e3 * float(np.percentile(times, 50)), "p99": 1e3 * float(np.percentile(times, 99))},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    barrier(world)


def run_batch_line(args):
    rank, world, local = dist_setup()
    from pixelflow_gb300 import _lib
    _lib.check(_lib.load().pf_set_device(local))
    r = bench_batch(ncases=args.cases, steps=args.steps, warmup_steps=max(1, args.warmup // 2))
    line = {"metric": METRIC, "value": r["value"] * world, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": r["workload"], "precision": "mixed", "form": "batched persistent kernel"},
            "batch": r, "gpu_launches": r["launches_in_timed_region"]}
    barrier(world)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_ours(args):
    if args.workload == "batch2d":
        return run_batch_line(args)
    rank, world, local = dist_setup()
    from pixelflow_gb300 import _lib
    from pixelflow_gb300.solver import Case, host_register, host_unregister
    _lib.check(_lib.load().pf_set_device(local))
    s, shape, vals, desc = workload(args.workload, args.precision)
    if args.precision == "mixed":
        s = s.replace(sweep_form=args.sweep_form)
        if args.schedule:
            o, i = (int(x) for x in args.schedule.lower().split("x"))
            s = s.replace(outer_max=o, inner_sweeps=i)
            desc.update(outer_passes=o, inner_sweeps=i)
    cells = int(np.prod(shape))
    case = Case(s, shape, vals)
    case.initial_conditions()
    case.step(args.warmup)
    case.synchronize()

    # ---- device-timed region ---------------------------------------------
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    case.synchronize()
    l0 = case.kernel_launches()
    case.profile_begin()
    case.step(args.steps)
    prof = case.profile_end()  # synchronizes the case's stream
    launches = case.kernel_launches() - l0
    barrier(world)
    clocks = sampler.stop()
    step_ms = reduce_max(prof["step_ms"], world)
    per_step = case.profile_step_times()
    stage_ms = case.profile_stages()
    value = world * cells * args.steps / (step_ms / 1e3) / 1e6
    max_div, sor_err = case.norms()
    # the plain state after warmup + steps, for the precision form's error below
    plain_state = case.get_state() if (args.forms and args.precision == "fp64") else None

    # ---- roofline of the dominant kernel (the red-black half-sweep) --------
    word = 8 if args.precision == "fp64" else 4
    sor_launch_ms = prof["sor_ms"] / max(prof["sor_launches"], 1)
    # algorithmic bytes per launch: the cells one launch updates (half of them
    # for a half-sweep, all of them for the fused full sweep of the precision
    # form) x 5 words (own p read, neighbour p read, p write, bb, porosity)
    sweeps = s.iter_max if args.precision == "fp64" else s.outer_max * s.inner_sweeps
    updates = cells * sweeps * prof["steps"] / max(prof["sor_launches"], 1)
    alg_bytes = updates * 5 * word
    achieved = alg_bytes / (sor_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    fused = args.precision == "mixed" and prof["sor_launches"] == sweeps * prof["steps"]
    listed = case.sor_info()["listed"]
    if args.precision == "fp64":
        kernel = "k_sor_list3" if listed else "k_sor_half"
        form = "sor_list" if listed else "sor_half"
    else:
        dc_listed = case.dc_list_info()["listed"]
        kernel = "k_sor_fused3" if fused else ("k_sor_dc_list3" if dc_listed else "k_sor_dc4")
        form = "sor_fused" if fused else ("sor_dc_list" if dc_listed else "sor_half")
    kname = f"{form}_{args.precision}_{args.workload}"
    traffic = ncu_traffic(kname)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": peak_kind, "kernel": kernel,
                "cell_updates_per_launch": updates,
                "sor_share_of_step": prof["sor_ms"] / prof["step_ms"], "avg_launch_ms": sor_launch_ms,
                "algorithmic_bytes_per_launch": alg_bytes}
    if args.precision == "fp64":
        # The FP64 roof (2 FMA/clk/SM on GB300): the reference's update is 7 FMAs
        # per cell (6 neighbours, the (1-w) p term) = 14 flops.  The list sweep
        # does 2 FMAs for a pure-fluid cell (the neighbour sum is exact integer
        # arithmetic), so its rate on the reference's flop count is "effective"
        # and can exceed the DGEMM roof.
        fp64_peak = fp64_peak_tflops()
        flops = cells / 2 * 14
        alu = flops / (sor_launch_ms / 1e3) / 1e12
        roofline["fp64_alu"] = {"achieved": alu, "peak": fp64_peak, "unit": "TFLOP/s", "frac": alu / fp64_peak,
                                "flops_per_launch": flops, "peak_source": "cuBLAS DGEMM 4096^3 measured live",
                                "counting": "effective (reference's 14 flops per update)" if listed else
                                            "executed"}
        if listed:
            roofline["binding"] = "hbm"
            roofline["fluid_cells"] = case.sor_info()["fluid"]
        else:
            roofline["binding"] = "fp64_alu" if alu / fp64_peak > achieved / peak else "hbm"

    # ---- end to end through the C ABI with host buffers ----------------------
    host = case.get_state()
    for a in host.values():
        host_register(a)
    out = {k: np.empty_like(a) for k, a in host.items()}
    for a in out.values():
        host_register(a)
    # pf_step_host: one step from host fields to host fields (input copies in
    # slabs beside the predictor); the same through the three calls it
    # stands for (set_state, step, get_state) for comparison.  Both are warmed
    # up first like the device-timed steps: the first pf_step_host call
    # allocates its staging, and the first step from each of the two
    # velocity buffers captures that buffer's step graph (one-time set-up),
    # so each form is warmed by consecutive calls covering both buffers.
    for _ in range(max(2, args.warmup)):
        case.step_host(host, out)
    for _ in range(max(2, args.warmup)):
        case.set_state(host["u"], host["v"], host["p"], host.get("w"))
        case.step(1)
        case.get_state(out)
    barrier(world)
    calls_a, calls_b = [], []
    # at least 40 calls (~1 s at 256^3); the per-call times are reported too
    # (on the shared box a call now and then stalls for 75-150 ms in either
    # form, the host side; the device-timed steps show no such outliers).
    # Python's cyclic garbage collector is off while the calls are timed: a
    # full collection of this process's heap (torch loaded) takes ~30 ms on
    # the machine's host, a pause of the measuring harness that the library's
    # own callers (a Fortran program through the C ABI) do not have.
    # Reference counting still frees everything the loop allocates.
    ncalls = max(args.steps, 40)
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    for _ in range(ncalls):
        ta = time.perf_counter()
        case.step_host(host, out)
        calls_a.append(1e3 * (time.perf_counter() - ta))
    t1 = time.perf_counter()
    e2e_s = reduce_max(t1 - t0, world)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(ncalls):
        ta = time.perf_counter()
        case.set_state(host["u"], host["v"], host["p"], host.get("w"))
        case.step(1)
        case.get_state(out)
        calls_b.append(1e3 * (time.perf_counter() - ta))
    t1 = time.perf_counter()
    three_s = reduce_max(t1 - t0, world)
    gc.enable()
    for a in list(host.values()) + list(out.values()):
        host_unregister(a)
    nbytes = sum(a.nbytes for a in host.values())
    e2e = {"value": world * cells * ncalls / e2e_s / 1e6, "unit": UNIT, "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes, "call": "pf_step_host", "calls": ncalls,
           "three_calls": world * cells * ncalls / three_s / 1e6,
           "per_call_ms": {"pf_step_host": {"median": statistics.median(calls_a), "min": min(calls_a),
                                            "max": max(calls_a), "all": [round(x, 2) for x in calls_a]},
                           "three_calls": {"median": statistics.median(calls_b), "min": min(calls_b),
                                           "max": max(calls_b), "all": [round(x, 2) for x in calls_b]}}}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic"}
    desc.update(parallelism=f"replicas{world}" if world > 1 else "single",
                l2="working set > 129 MB L2 (no flush needed)")
    line["config"] = desc
    line["latency_ms"] = {"p50": float(np.percentile(per_step, 50)), "p99": float(np.percentile(per_step, 99))}
    line["max_div"] = max_div
    line["sor_error"] = sor_err
    line["roofline"] = roofline
    line["stages"] = stage_roofline(stage_ms, prof["steps"], cells, len(shape), s, args.precision, peak, peak_kind)
    line["e2e"] = e2e
    line["gpu_launches"] = launches
    line["clocks"] = clocks
    case.close()
    if args.forms and args.precision == "fp64" and args.workload.startswith("spheres3d"):
        # the precision form on the same case (the FP32 sweep's form and tile
        # and the outer x inner schedule, at most 4 passes of 25 sweeps, from
        # the autotuner, which also reports every candidate's speed and
        # error), and the batched form (2D batch)
        from pixelflow_gb300.autotune import tune_fused, tune_schedule
        ms_ = s.replace(precision="mixed")
        tile, tile_trials = tune_fused(ms_, shape, vals, use_cache=False)
        sched, sched_trials = tune_schedule(ms_, shape, vals, bound=args.schedule_bound, use_cache=False)
        mc = Case(ms_.replace(outer_max=sched[0], inner_sweeps=sched[1], **tile), shape, vals)
        mc.initial_conditions()
        mc.step(args.warmup)
        mc.synchronize()
        mc.profile_begin()
        mc.step(args.steps)
        mp = mc.profile_end()
        mdiv, _ = mc.norms()
        mstate = mc.get_state()
        msweep = mc.sweep_info()
        mc.close()
        # relative L2 of the precision form against the plain FP64 run after the
        # same number of steps from the same initial state (interior cells)
        inner = tuple(slice(1, -1) for _ in range(len(shape)))
        err = {}
        for f in plain_state:
            a, b = mstate[f][inner], plain_state[f][inner]
            err[f] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
        mval = world * cells * args.steps / (reduce_max(mp["step_ms"], world) / 1e3) / 1e6
        line["forms"] = {"mixed_same_case": {"value": mval, "unit": UNIT, "max_div": mdiv,
                                             "speedup_vs_plain_fp64": mval / value,
                                             "rel_l2_vs_fp64": err, "after_steps": args.warmup + args.steps,
                                             "schedule": f"{sched[0]} passes x {sched[1]} FP32 sweeps, "
                                                         "FP64 residual/accumulation",
                                             "sweep": msweep,
                                             "autotune": {"tile": tile, "tile_trials": tile_trials,
                                                          "schedule_bound": args.schedule_bound,
                                                          "schedule_pick": list(sched),
                                                          "schedule_trials": sched_trials}}}
        if not args.no_batch:
            line["forms"]["batch2d_512"] = bench_batch(steps=args.steps, plain_value=value,
                                                       schedule_bound=args.schedule_bound)
            line["forms"]["serving"] = bench_serving(policy="srpt_fill", plain_value=value,
                                                     schedule_bound=args.schedule_bound)
            line["forms"]["serving_round_robin"] = bench_serving(policy="rr", baseline_steps=0,
                                                                 schedule_bound=args.schedule_bound)
            if args.serving_rates:
                rates = tuple(float(x) for x in args.serving_rates.split(","))
                line["forms"]["serving_rates"] = bench_serving_rates(rates, count=args.rate_requests,
                                                                     schedule_bound=args.schedule_bound)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(s.replace(precision="fp64"), shape, vals)
    barrier(world)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="spheres3d_256")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--sweep-form", default="auto", choices=["auto", "split", "fused"],
                    help="precision form: the FP32 sweep's form (auto: timed on the case at creation)")
    ap.add_argument("--schedule", default="",
                    help="precision form: outer passes x FP32 sweeps per pass, e.g. 1x100 (default: 4x25)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--forms", type=int, default=1, help="also measure the precision and batched forms")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--cases", type=int, default=512, help="batch2d workload: number of 2D cases")
    ap.add_argument("--serving-rates", default="0.5,1,2",
                    help="serving form at these arrival rates (requests/s); empty to skip")
    ap.add_argument("--rate-requests", type=int, default=32, help="requests per arrival rate")
    ap.add_argument("--schedule-bound", type=float, default=1e-6,
                    help="precision form: the autotuner's bound on the relative L2 error against FP64 when it "
                         "picks the outer x inner schedule")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
