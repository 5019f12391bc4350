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

--impl reference times the FP64 oracle (the CPU restatement of the
reference's kinetic path; no Fortran compiler exists on either machine) on
the same workload, full velocity grid included, on all host cores.
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
# what the mixed path computes in which type
PREC_MIXED = ("fp32 f, fluxes, equilibrium and sweeps; moments: fp32 products summed in fp32 over blocks of 16 "
              "velocities (8 on rows the packed pass does not take), the blocks Kahan-compensated in fp32, "
              "velocity slices folded in float-float, the primitive conversion and residual in fp64")
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
def cpu_oracle(case, threads):
    """The FP64 oracle (CPU restatement of the reference path) on the same
    mesh and the same full velocity grid as the GPU run."""
    from oracle import oracle as O
    import copy
    c = copy.deepcopy(case)
    c.precision = 0
    o = O.Oracle(c, threads=threads)
    o.init_maxwellian()
    return c, o


def cpu_sample(case, seconds=10.0, threads=0, oracle=None):
    """Cell-velocity updates/s of the oracle on the full workload, over whole
    iterations until `seconds` have passed (at least one)."""
    nthreads = threads or (os.cpu_count() or 1)
    if oracle is None:
        c, o = cpu_oracle(case, nthreads)
    else:
        c, o = oracle
        from oracle import oracle as O
        O.lib().orc_set_threads(nthreads)
    n = 0
    t0 = time.perf_counter()
    while True:
        o.step(1)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    val = c.cells * c.nv * n / el
    return val, nthreads, (f"{c.ncx}x{c.ncy} cells x {c.nvx}x{c.nvy} velocities (the full workload), "
                           f"{n} FP64 oracle iterations, {el:.1f}s")


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


class PinnedArray:
    """A float64 host array in page-locked memory (cudaHostAlloc through the
    CUDA runtime the library already loaded): the end-to-end leg reads the
    step's results into it, as a host that keeps its output fields pinned."""

    def __init__(self, n):
        import ctypes as C
        self.rt = None
        for name in ("libcudart.so.13", "libcudart.so"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        if self.rt is None:
            raise RuntimeError("CUDA runtime library not found")
        self.rt.cudaHostAlloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t, C.c_uint]
        self.rt.cudaFreeHost.argtypes = [C.c_void_p]
        self.p = C.c_void_p()
        if self.rt.cudaHostAlloc(C.byref(self.p), n * 8, 0) != 0:
            raise RuntimeError("cudaHostAlloc failed")
        self.a = np.ctypeslib.as_array((C.c_double * n).from_address(self.p.value))

    def free(self):
        if self.p:
            self.a = None
            self.rt.cudaFreeHost(self.p)
            self.p = None


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
    (the Fortran reference has no compiler here) on the machine's host cores, on
    the same mesh and velocity grid as the GPU arm."""
    if rank != 0:
        return 0
    case = make_case(args.config)
    nthreads = os.cpu_count() or 1
    c, o = cpu_oracle(case, nthreads)
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
                   "sample": "the full workload: same mesh, same velocity grid, one outer iteration per step"},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{c.ncx}x{c.ncy} cells x {c.nvx}x{c.nvy} velocities per step, FP64 oracle, "
                                   f"{nthreads} OpenMP threads"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _ttr_run(name, case, prec, gsis=None, promote=False, learned=False, tol=1e-8, max_iters=8000, chunk=50,
             wall_s=None, finish_below=None, finish_gsis=None):
    """One run to max RMS residual <= tol (DETFP_res): device-synchronised
    wall clock around the hyb_step calls, the residual read every `chunk`
    outer iterations.  promote: a mixed run continues in FP64 on the device
    (hyb_set_precision) once its FP32 residual stops falling.  An FP32 run
    without promotion that has not improved for 1000 iterations below 1e-4
    sits on its rounding floor and is stopped.  wall_s caps the wall time.
    finish_below, finish_gsis: a synthetic-solve run whose residual, below
    finish_below, has fallen by less than 10 % over the last three
    checkpoints (and, with promote, after the promotion) is reconfigured
    with finish_gsis (hyb_gsis_configure; {"enable": 0} for the plain
    iteration).  The coupled iteration can settle on a fixed point of its
    own a little off the kinetic one: with the distribution correction on,
    its residual stops falling there, and it falls again once only the
    moments are corrected."""
    from hyb_gb300 import closure, hyb_types as T
    s = abi.Solver(case, precision=prec)
    s.init_maxwellian()
    if gsis is not None:
        if learned:
            s.attach_mlp(closure.load())
        s.gsis(**gsis)
    it, r, prev, promoted, best, best_it, stalled = 0, None, None, None, None, 0, False
    finished = None
    hist = []
    t0 = time.perf_counter()
    while it < max_iters:
        r = s.step(chunk)
        it += chunk
        res = r["max_rms"]
        hist.append([it, float("%.3g" % res)])
        if res <= tol or not np.isfinite(res):
            break
        if wall_s is not None and time.perf_counter() - t0 > wall_s:
            break
        if best is None or res < 0.9 * best:
            best, best_it = res, it
        elif prec == T.HYB_PREC_MIXED and not promote and res < 1e-4 and it - best_it >= 1000:
            stalled = True
            break
        if promote and promoted is None and prev is not None and res < 1e-3 and res > 0.9 * prev:
            s.set_precision(T.HYB_PREC_FP64)
            promoted = it
        elif (finish_below is not None and gsis is not None and finished is None and res < finish_below
              and (promoted is not None or not promote) and len(hist) > 3 and res > 0.9 * hist[-4][1]):
            s.gsis(**finish_gsis)
            finished = it
        prev = res
    el = time.perf_counter() - t0
    S = s.moments()[0].reshape(case.ny + 7, case.nx + 7, 11)[4:4 + case.ny - 1, 4:4 + case.nx - 1, :4]
    out = {"seconds": round(el, 3), "iterations": it, "ms_per_iteration": round(1000.0 * el / it, 3),
           "residual": r["max_rms"], "reached": bool(r["max_rms"] <= tol),
           "precision": "mixed" if prec == T.HYB_PREC_MIXED else "fp64", "history": hist}
    if promote:
        out["fp64_from_iteration"] = promoted
    if finish_below is not None:
        out["finish_from_iteration"] = finished
    if stalled:
        out["stalled_on_fp32_floor"] = True
    if gsis is not None:
        out["skipped_corrections"] = s.gsis_skipped()
    s.close()
    return out, S


def time_to_residual(tol=1e-8, large=True):
    """Time to residual 1e-8.  The Kn 0.1 channel (4x64 cells, 32^2 NC,
    plates +-0.2): the reference's own iteration (forward sweep in index
    order with the Jacobi-like backward step, dt 0.01), the upwind-ordered
    iteration at dt 1e6 with the mass pin, and the synthetic-solve variants,
    each FP64 and mixed (finished in FP64 on the device).  The large case
    (128x512 cells, 64^2 on [-6,6], Kn 0.01): the synthetic solve with the
    line-averaged correction in FP64, mixed finished in FP64, and mixed with
    the learned warm start finished in FP64, each to 1e-8 within 400 outer
    iterations and 100 s; beside them the synthetic solve without the
    line-averaged correction and the plain iteration, each for a bounded
    number of iterations.  Field differences are stated against the FP64 run
    of the same iteration."""
    from hyb_gb300 import hyb_types as T
    M, D = T.HYB_PREC_MIXED, T.HYB_PREC_FP64
    ref = lambda: cases.couette_small(dt=0.01)
    upw = lambda: cases.couette_small(dt=1.0e6, sweep_order=1, mass_pin=1)
    gs = dict(max_inner=40, inner_tol=0.0, inner_rtol=1e-2, cfl=20.0, ns_solver=0, correct_f=1)
    gl = dict(gs, mlp_warm_after=20, mlp_warm_inner=400)
    small = [("plain_fp64_reference_iteration", ref, D, None, False, False),
             ("plain_mixed_reference_iteration_to_fp64", ref, M, None, True, False),
             ("plain_fp64_upwind", upw, D, None, False, False),
             ("plain_mixed_upwind_to_fp64", upw, M, None, True, False),
             ("gsis_fp64", ref, D, gs, False, False),
             ("gsis_mixed_to_fp64", ref, M, gs, True, False),
             ("gsis_mixed_learned_to_fp64", ref, M, gl, True, True)]
    out, fields = {}, {}
    for name, mk, prec, g, promote, learned in small:
        out[name], fields[name] = _ttr_run(name, mk(), prec, g, promote, learned, tol=tol)
    # field error of each run against the FP64 run of the same iteration
    base = {"reference": fields["plain_fp64_reference_iteration"], "upwind": fields["plain_fp64_upwind"],
            "gsis": fields["gsis_fp64"]}
    for name, S in fields.items():
        b = base["upwind" if "upwind" in name else ("gsis" if name.startswith("gsis") else "reference")]
        out[name]["field_rel_err_vs_fp64"] = {
            k: float(np.abs(S[..., q] - b[..., q]).max() / max(np.abs(b[..., q]).max(), 1e-3))
            for q, k in enumerate(("rho", "u", "v", "T"))}
    res = {"workload": "couette-4x64-nv32-kn0.1, NND", "tol": tol, "runs": out}
    if large:
        gl2 = dict(wall_band=1, correct_f=1, ns_solver=2, cfl=600.0, max_inner=16, inner_tol=0.0,
                   inner_rtol=1e-8, relax_pct=70)
        glm = dict(gl2, line_mean=1)
        lg, fl = {}, {}
        # (name, precision, outer-iteration cap, synthetic solve, residual chunk, promote, learned)
        runs = (("gsis_fp64_line_mean", D, 400, glm, 10, False, False),
                ("gsis_mixed_line_mean_to_fp64", M, 400, glm, 10, True, False),
                ("gsis_mixed_learned_line_mean_to_fp64", M, 400, dict(glm, mlp_warm_after=20, mlp_warm_inner=400),
                 10, True, True),
                ("gsis_mixed_without_line_mean", M, 150, gl2, 10, False, False),
                ("plain_mixed", M, 600, None, 50, False, False))
        for name, prec, cap, g, chunk, promote, learned in runs:
            c = cases.couette_large(dt=1.0e6, sweep_order=1, mass_pin=1, precision=prec)
            lg[name], fl[name] = _ttr_run(name, c, prec, g, promote, learned, tol=tol, max_iters=cap, chunk=chunk,
                                          wall_s=100.0)
        b = fl["gsis_fp64_line_mean"]
        for name in ("gsis_mixed_line_mean_to_fp64", "gsis_mixed_learned_line_mean_to_fp64"):
            S = fl[name]
            lg[name]["field_rel_err_vs_fp64"] = {
                k: float(np.abs(S[..., q] - b[..., q]).max() / max(np.abs(b[..., q]).max(), 1e-3))
                for q, k in enumerate(("rho", "u", "v", "T"))}
            if lg[name]["reached"] and lg["gsis_fp64_line_mean"]["reached"]:
                lg[name]["wall_time_ratio_fp64_over_this"] = (lg["gsis_fp64_line_mean"]["seconds"] /
                                                               lg[name]["seconds"])
        res["large"] = {"workload": "couette-128x512-nv64-kn0.01, upwind order dt 1e6, mass pin; GSIS band to "
                                    "the walls, line solver (16 inner, CFL 600) with the line-averaged "
                                    "correction, correction relaxed to 0.7; the same without the line-averaged "
                                    "correction and the plain iteration of the same order for comparison",
                        "cap_iterations": {"gsis": 400, "gsis_without_line_mean": 150, "plain": 600},
                        "cap_seconds": 100.0, "runs": lg}
    return res


def time_to_residual_sine():
    """The 512x512 sine case (48^2 on [-5, 5], Kn 0.005, T_w = 1 + 0.1 sin(2 pi x),
    plates +-0.3), mixed precision, upwind order at dt 1e6 with the mass pin:
    the plain iteration for 1000 iterations; the synthetic solve with the
    line-averaged correction and its first two harmonics, with and without
    the learned warm start, and with the constant mode only, for 400 outer
    iterations each; the synthetic solve without the correction for 150; and
    the synthetic solve with the harmonics and the unlimited NND stencil,
    promoted to FP64 at its FP32 floor and reconfigured to correct the
    moments only at its own floor, to 1e-8 within 1000 outer iterations and
    300 s.  The mixed runs stop on their
    FP32 floor, so they report the residual each reaches and the cost of an
    iteration."""
    from hyb_gb300 import hyb_types as T
    M = T.HYB_PREC_MIXED
    gl2 = dict(wall_band=1, correct_f=1, ns_solver=2, cfl=600.0, max_inner=16, inner_tol=0.0, inner_rtol=1e-8,
               relax_pct=70)
    glm = dict(gl2, line_mean=1)
    glh = dict(gl2, line_mean=3)
    # the finishing run: the unlimited NND stencil in the synthetic equation,
    # and the moments-only correction once the coupled iteration stalls
    glf = dict(glh, ns_scheme=2)
    out = {}
    # (name, synthetic solve, learned, outer-iteration cap, chunk, promote to FP64 and hand over to the
    # plain iteration at its floor)
    for name, g, learned, cap, chunk, finish in (
            ("plain_mixed", None, False, 1000, 50, False),
            ("gsis_mixed_harmonics", glh, False, 400, 10, False),
            ("gsis_mixed_learned_harmonics", dict(glh, mlp_warm_after=20, mlp_warm_inner=400), True, 400, 10, False),
            ("gsis_mixed_line_mean", glm, False, 400, 10, False),
            ("gsis_mixed_without_line_mean", gl2, False, 150, 10, False),
            ("gsis_mixed_harmonics_to_fp64_then_moments_only", glf, False, 1000, 10, True)):
        c = cases.couette_sine(dt=1.0e6, sweep_order=1, mass_pin=1, precision=M)
        out[name], _ = _ttr_run(name, c, M, g, finish, learned, tol=1e-8, max_iters=cap, chunk=chunk,
                                wall_s=300.0 if finish else None, finish_below=1e-6 if finish else None,
                                finish_gsis=dict(g, correct_f=0) if finish else None)
    return {"workload": "couette-512x512-nv48-kn0.005-sine, upwind order dt 1e6, mass pin", "runs": out}


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
    S_pin, cf_pin = PinnedArray(11 * (case.nx + 7) * (case.ny + 7)), PinnedArray((case.nx + 3) * (case.ny + 3))
    S_host, cf_host = S_pin.a, cf_pin.a
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
    S_host = cf_host = None
    S_pin.free()
    cf_pin.free()
    s.close()
    # ---- the same workload through the FP64 path ------------------------------
    fp64 = None
    if case.precision == 1 and not args.no_fp64:
        import copy
        c64 = copy.deepcopy(case)
        c64.precision = 0
        s64 = abi.Solver(c64, device=local)
        s64.init_maxwellian()
        for _ in range(args.warmup):
            s64.step(1, residual=False)
        s64.profile(True)
        dist_barrier(world)
        n64 = max(3, args.steps // 4)
        s64.step(n64, residual=False)
        ms64 = dist_max(world, s64.last_ms())
        p64 = s64.profile_read()
        s64.close()
        fp64 = {"value": world * case.cells * case.nv * n64 / (ms64 / 1000.0), "unit": UNIT, "steps": n64,
                "ms_per_step": ms64 / n64, "dtype": "f64",
                "stage_ms_per_step": {k: round(v_[0] / n64, 4) for k, v_ in p64.items() if v_[1]},
                "note": "GB300 issues FP64 at 2 lanes per clock per SM: the FP64 sweep is bound by FP64 "
                        "arithmetic, not by HBM"}
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
                   "precision": PREC_MIXED if case.precision == 1 else "fp64",
                   "scheme": "NND", "dt": case.dt, "parallelism": f"replicas x{world}",
                   "sweep_shape": {"cells_per_thread": shape[0], "velocities_per_cta": shape[1]},
                   "l2": "inputs larger than L2 (f is %.2f GB)" % (case.cells * case.nv * 2 * rs / 1e9)},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "calls": "hyb_set_walls x2 + hyb_step(1, residual) + hyb_download_moments per step",
                "host_buffers": "moments and CF read into page-locked host arrays; wall data staged by the "
                                "library through its page-locked buffer"},
        "roofline": {"bound": "hbm", "kernel": "k_sweep", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind, "alg_bytes_per_cell_velocity": b_alg,
                     "ms_per_launch": per_launch_s * 1000.0},
        "whole_step": {"bytes_per_unit": 6 * rs,
                       "note": "bytes the step moves per cell-velocity: the fused sweep reads and writes G, H "
                               "(4 s), the moment pass reads them (2 s)",
                       "achieved_gbs": 6 * rs * units / (ms / 1000.0) / 1e9 / world,
                       "frac": 6 * rs * units / (ms / 1000.0) / 1e9 / world / peak},
        "stage_ms_per_step": stage_ms,
        "gpu_launches": launches,
        "clocks": clk,
        "last_residual": res["max_rms"],
    }
    if fp64 is not None:
        line["fp64"] = fp64
    # the convergence runs are reported beside the throughput line: an error
    # in one of them is recorded in its key and does not lose the line
    if not args.no_ttr and rank == 0:
        try:
            line["time_to_residual"] = time_to_residual(large=not args.no_ttr_large)
        except Exception as e:   # noqa: BLE001
            line["time_to_residual"] = {"error": f"{type(e).__name__}: {e}"}
    if args.ttr_sine and rank == 0:
        try:
            line["time_to_residual_sine"] = time_to_residual_sine()
        except Exception as e:   # noqa: BLE001
            line["time_to_residual_sine"] = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_cpu:
        orc = cpu_oracle(case, os.cpu_count() or 1)
        orc[1].step(1)
        cv, cores, sample = cpu_sample(case, seconds=args.cpu_seconds, oracle=orc)
        cv1, _, sample1 = cpu_sample(case, seconds=1.0, threads=1, oracle=orc)
        del orc
        line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                                "value_1_thread": cv1, "sample_1_thread": sample1,
                                "nproc": os.cpu_count(), "cpu_model": cpu_model()}
        # the channel to 1e-8 on the host: oracle time per iteration times
        # the plain iteration count measured on the GPU (FP64 parity makes
        # the two runs take the same iterations)
        it_s = cpu_channel_iteration_s()
        ttr = line.get("time_to_residual", {}).get("runs", {}).get("plain_fp64_reference_iteration")
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
    ap.add_argument("--no-ttr-large", action="store_true", help="time to residual on the small channel only")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 throughput of the same workload")
    ap.add_argument("--ttr-sine", action="store_true",
                    help="add the bounded residual runs of the 512x512 sine case (about 20 s)")
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
