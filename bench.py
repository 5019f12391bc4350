"""Benchmark of the GB300 kinetic hot path: one outer iteration = one step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--config large|small|sine]

Default workload (config "large"): single planar Couette, 128x512 cells,
64x64 Newton-Cotes velocity grid on [-6,6], Kn=0.01, plates at +-0.5,
wall temperatures 1.0 / 1.2, FP32 distribution with FP64 moments.  The metric
is cell-velocity updates per second (cells x velocity nodes x iterations /
time).  Inputs (f, 2.1 GB) are larger than L2, so no flush is needed between
steps.  N > 1 runs independent replicas, one per GPU (the path is not
sharded across GPUs); value is the sum over ranks.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as GE  # noqa: E402

GE.load_package()
from hyb_gb300 import abi, cases  # noqa: E402

METRIC = "cell-velocity updates/s (plain kinetic iteration)"
UNIT = "cell*velocity updates/s"


def make_case(name):
    if name == "large":
        return cases.couette_large(dt=0.00625)
    if name == "sine":
        return cases.couette_sine(dt=0.00625)
    if name == "prof":   # profiling case: the large mesh with a 24x24 grid (f = 302 MB > L2)
        return cases.couette_large(dt=0.00625, nvx=24, nvy=24)
    return cases.couette_small(dt=0.05)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY, "--format=csv,noheader",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1].split()[0]))
                smax.append(float(p[2].split()[0]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def cpu_sample(case, seconds=10.0, max_seconds=30.0, threads=0):
    """Oracle (CPU restatement of the reference path) on the same mesh with a
    16x16 velocity subset; returns cell-velocity updates/s and the sample."""
    from oracle import oracle as O
    import copy
    c = copy.deepcopy(case)
    c.nvx = c.nvy = 16
    c.precision = 0
    nthreads = threads or (os.cpu_count() or 1)
    o = O.Oracle(c, threads=nthreads)
    o.init_maxwellian()
    o.step(1)
    n = 0
    t0 = time.perf_counter()
    while True:
        o.step(1)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or el >= max_seconds:
            break
    val = c.cells * c.nv * n / el
    return val, nthreads, f"{c.ncx}x{c.ncy} cells x 16x16 velocities, {n} FP64 oracle iterations, {el:.1f}s"


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.machine()


def cpu_channel_iteration_s(seconds=3.0):
    """Oracle seconds per plain FP64 iteration of the Kn 0.1 channel (4x64
    cells, 32x32 velocities) on all host cores."""
    from oracle import oracle as O
    o = O.Oracle(cases.couette_small(dt=0.01), threads=os.cpu_count() or 1)
    o.init_maxwellian()
    o.step(1)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        o.step(10)
        n += 10
    return (time.perf_counter() - t0) / n


# ---------------------------------------------------------------------------
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(world, x):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def run_reference(args, world, rank):
    """The reference arm: the CPU restatement of the reference's kinetic path
    (the Fortran reference has no compiler here) on the machine's host cores."""
    if rank != 0:
        return 0
    case = make_case(args.config)
    from oracle import oracle as O
    import copy
    c = copy.deepcopy(case)
    c.nvx = c.nvy = 16
    c.precision = 0
    nthreads = os.cpu_count() or 1
    o = O.Oracle(c, threads=nthreads)
    o.init_maxwellian()
    for _ in range(args.warmup):
        o.step(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(1)
    el = time.perf_counter() - t0
    val = c.cells * c.nv * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": case.name, "cells": case.cells, "velocities": case.nv,
                   "sample": f"same mesh, 16x16 velocity subset per step"},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{c.ncx}x{c.ncy} cells x 16x16 velocities per step, FP64 oracle, "
                                   f"{nthreads} OpenMP threads"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def time_to_residual(tol=1e-8, max_iters=8000, chunk=50):
    """Wall time and outer iterations to max RMS residual <= tol on the Kn 0.1
    channel (4x64 cells, 32x32 NC, NND, dt 0.01), for the plain kinetic
    iteration and the synthetic-solve variants; device-synchronised wall
    clock around the hyb_step calls (residual read every `chunk` steps)."""
    from hyb_gb300 import closure
    gs = dict(max_inner=40, inner_tol=0.0, inner_rtol=1e-2, cfl=20.0, ns_solver=0, correct_f=1)
    # "switch" variants run FP32 f until the residual reaches `switch_at`
    # (or stops falling) and continue the same state in an FP64 context
    # the learned warm start after 20 outer iterations, 400 inner iterations
    # of the closed NS equations (2000 cost more than they saved)
    gl = dict(gs, mlp_warm_after=20, mlp_warm_inner=400)
    variants = [("plain_fp64", 0, None, False), ("gsis_fp64", 0, gs, False), ("gsis_mixed", 1, gs, False),
                ("gsis_mixed_learned", 1, gl, False),
                ("gsis_mixed_then_fp64", 1, gs, True), ("gsis_mixed_learned_then_fp64", 1, gl, True)]
    net = closure.load()
    out = {}
    switch_at = 3e-6
    for name, prec, g, switch in variants:
        c = cases.couette_small(dt=0.01)
        s = abi.Solver(c, precision=prec)
        s.init_maxwellian()
        if g is not None:
            s.attach_mlp(net)
            s.gsis(**g)
        it, r, prev, switched_at = 0, None, None, None
        best, best_it, stalled = None, 0, False
        t0 = time.perf_counter()
        while it < max_iters:
            r = s.step(chunk)
            it += chunk
            if r["max_rms"] <= tol:
                break
            # an FP32 run that has stopped falling below 1e-4 for 1000
            # iterations sits on its rounding floor: stop and report it
            if best is None or r["max_rms"] < 0.9 * best:
                best, best_it = r["max_rms"], it
            elif prec == 1 and not switch and r["max_rms"] < 1e-4 and it - best_it >= 1000:
                stalled = True
                break
            if switch and switched_at is None and (r["max_rms"] <= switch_at or (
                    r["max_rms"] < 1e-4 and prev is not None and r["max_rms"] > 0.9 * prev)):
                f = s.download_f()
                s.close()
                s = abi.Solver(c, precision=0)
                s.upload_f(f)
                s.gsis(**{k: v for k, v in g.items() if k != "mlp_warm_after"})
                switched_at = it
            prev = r["max_rms"]
        el = time.perf_counter() - t0
        u = s.moments()[0].reshape(c.ny + 7, c.nx + 7, 11)[4:4 + c.ny - 1, 4:4 + c.nx - 1, 1]
        out[name] = {"seconds": round(el, 3), "iterations": it, "residual": r["max_rms"],
                     "reached": bool(r["max_rms"] <= tol), "u_mid_wall": float(u[-1].mean())}
        if switch:
            out[name]["fp64_from_iteration"] = switched_at
        if stalled:
            out[name]["stalled_on_fp32_floor"] = True
        s.close()
    ref = out["plain_fp64"]["u_mid_wall"]
    for v in out.values():
        v["u_wall_rel_diff_vs_plain"] = abs(v["u_mid_wall"] - ref) / abs(ref)
    return {"workload": "couette-4x64-nv32-kn0.1, NND, dt 0.01", "tol": tol, "chunk": chunk, "runs": out}


def run_gb300(args, world, rank, local):
    case = make_case(args.config)
    s = abi.Solver(case, device=local)
    s.init_maxwellian()
    shape = s.autotune(reps=3)                # sweep launch shape picked by timing
    for _ in range(args.warmup):
        s.step(1, residual=False)
    # ---- device-timed region ------------------------------------------------
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    s.profile(True)
    l0 = s.launches()
    dist_barrier(world)
    s.step(args.steps, residual=False)        # events on the library's stream
    ms = s.last_ms()
    launches = s.launches() - l0
    prof = s.profile_read()
    s.profile(False)
    dist_barrier(world)
    clk = clocks.stop()
    ms = dist_max(world, ms)
    units = case.cells * case.nv * args.steps
    value = world * units / (ms / 1000.0)
    # ---- roofline of the dominant kernel (the fused sweep) ---------------------
    rs = 4 if case.precision == 1 else 8
    b_alg = 2 * 2 * rs                        # read G,H and write G,H per cell-velocity
    sweep_ms, sweep_n = prof["sweep"]
    per_launch_s = sweep_ms / 1000.0 / max(sweep_n, 1)
    achieved = b_alg * case.cells * case.nv / per_launch_s / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "sweep_traffic.json")
    if os.path.exists(tfile):
        with open(tfile) as fh:
            t = json.load(fh)
        if t.get("workload") == case.name and t.get("precision") == case.precision:
            traffic = t.get("bytes_per_launch")
    # ---- end to end through the C ABI with host buffers ------------------------
    u, v, t = case.walls()
    S_host = np.zeros(11 * (case.nx + 7) * (case.ny + 7))
    cf_host = np.zeros((case.nx + 3) * (case.ny + 3))
    h2d = sum(3 * 8 * len(u[f]) for f in (1, 3))
    d2h = S_host.nbytes + cf_host.nbytes + 9 * 8
    dist_barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for f in (1, 3):
            s.set_walls(f + 1, u[f], v[f], t[f])
        res = s.step(1, residual=True)
        s.L.hyb_download_moments(s.h, S_host.ctypes.data_as(abi.C.POINTER(abi.C.c_double)),
                                 cf_host.ctypes.data_as(abi.C.POINTER(abi.C.c_double)))
    e2e_s = dist_max(world, time.perf_counter() - t0)
    e2e = world * units / e2e_s
    s.close()
    if rank != 0:
        return 0
    stage_ms = {k: round(v_[0] / args.steps, 4) for k, v_ in prof.items() if v_[1]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if case.precision == 1 else "f64",
        "data": "synthetic (seeded analytic Couette set-up; no dataset)",
        "config": {"workload": case.name, "cells": case.cells, "velocities": case.nv,
                   "precision": "fp32 f/fluxes/sweeps, fp64 moments" if case.precision == 1 else "fp64",
                   "scheme": "NND", "dt": case.dt, "parallelism": f"replicas x{world}",
                   "sweep_shape": {"cells_per_thread": shape[0], "velocities_per_cta": shape[1]},
                   "l2": "inputs larger than L2 (f is %.2f GB)" % (case.cells * case.nv * 2 * rs / 1e9)},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "calls": "hyb_set_walls x2 + hyb_step(1, residual) + hyb_download_moments per step"},
        "roofline": {"bound": "hbm", "kernel": "k_sweep", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind, "alg_bytes_per_cell_velocity": b_alg,
                     "ms_per_launch": per_launch_s * 1000.0},
        "whole_step_basis": {"bytes_per_unit": 40, "note": "whole kinetic step on the 5*NRD*s definition",
                         "achieved_gbs": 40.0 * units / (ms / 1000.0) / 1e9 / world,
                         "frac": 40.0 * units / (ms / 1000.0) / 1e9 / world / peak},
        "stage_ms_per_step": stage_ms,
        "gpu_launches": launches,
        "clocks": clk,
        "last_residual": res["max_rms"],
    }
    if not args.no_ttr and rank == 0:
        line["time_to_residual"] = time_to_residual()
    if not args.no_cpu:
        cv, cores, sample = cpu_sample(case, seconds=args.cpu_seconds)
        cv1, _, sample1 = cpu_sample(case, seconds=args.cpu_seconds / 2, threads=1)
        line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                                "value_1_thread": cv1, "sample_1_thread": sample1,
                                "nproc": os.cpu_count(), "cpu_model": cpu_model()}
        # the channel to 1e-8 on the host: oracle time per iteration times
        # the plain iteration count measured on the GPU (FP64 parity makes
        # the two runs take the same iterations)
        it_s = cpu_channel_iteration_s()
        ttr = line.get("time_to_residual", {}).get("runs", {}).get("plain_fp64")
        line["cpu_baseline"]["channel_plain_fp64_s_per_iteration"] = it_s
        if ttr and ttr.get("reached"):
            line["cpu_baseline"]["channel_plain_fp64_to_1e-8_s_extrapolated"] = it_s * ttr["iterations"]
    print(json.dumps(line), flush=True)
    return 0


def batch_cases():
    """The seeded 256-instance manifest, FP32 distribution, dt scaled with the
    cell size (kinetic CFL about 3 for the 64-cell channel at dt 0.01)."""
    out = []
    for d in cases.batch_manifest():
        out.append(cases.Case(precision=1, dt=0.01 * 64.0 / d["ncy"], **d))
    return out


def run_batch(args, world, rank, local):
    # one hardware queue per concurrent graph branch, up to the device limit;
    # read when the CUDA context is created, so set before the first call
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    cl = batch_cases()
    b = abi.Batch(cl, device=local)
    b.init_maxwellian()
    t_tune = time.perf_counter()
    b.autotune(reps=2)
    t_tune = time.perf_counter() - t_tune
    b.step(args.warmup, residual=False)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    l0 = b.launches()
    dist_barrier(world)
    b.step(args.steps, residual=False)
    ms = b.last_ms()
    launches = b.launches() - l0
    dist_barrier(world)
    clk = clocks.stop()
    ms = dist_max(world, ms)
    units = sum(c.cells * c.nv for c in cl) * args.steps
    value = world * units / (ms / 1000.0)
    # the same iterations issued instance by instance through hyb_step
    views = [b.instance(k) for k in range(len(cl))]
    t0 = time.perf_counter()
    for v_ in views:
        v_.step(args.steps, residual=False)
    seq_ms = 1000.0 * (time.perf_counter() - t0)
    # end to end: residuals of every instance read back each step
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = b.step(1, residual=True)
    e2e_s = dist_max(world, time.perf_counter() - t0)
    peak, peak_kind = measured_peaks()
    achieved = 16.0 * units / args.steps / (ms / args.steps / 1000.0) / 1e9
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded instance manifest, default_rng(20261203))",
        "config": {"workload": "batched Couette, 256 instances", "instances": len(cl),
                   "cell_velocities_per_step": units // args.steps,
                   "precision": "fp32 f/fluxes/sweeps, fp64 moments", "scheme": "NND",
                   "launch": "one CUDA graph launch per outer iteration; one batched launch per kernel and "
                             "launch-shape group (instances grouped by sweep shape)",
                   "autotune_s": round(t_tune, 2), "parallelism": f"replicas x{world}",
                   "l2": "per-step working set above L2 (sum of f over instances)"},
        "e2e": {"value": world * units / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": len(cl) * 9 * 8,
                "calls": "hyb_batch_step(1) with every instance's residual read back"},
        "roofline": {"bound": "hbm", "kernel": "whole batched step (16 B per cell-velocity)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_kind": peak_kind},
        "sequential_ms_per_step": seq_ms / args.steps,
        "graph_speedup_vs_sequential": seq_ms / ms,
        "gpu_launches": launches,
        "clocks": clk,
        "last_residual_max": max(r["max_rms"] for r in res),
    }
    print(json.dumps(line), flush=True)
    b.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="large", choices=["large", "small", "sine", "prof", "batch"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ttr", action="store_true", help="skip the time-to-residual runs")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_init()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.config == "batch":
        return run_batch(args, world, rank, local)
    return run_gb300(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
