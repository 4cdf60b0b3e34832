"""Benchmark of the projection-step pressure solve on GB300.

Headline metric: Poisson solves/s at ||r||/||b|| = 1e-10 on the 512^3
mixed-precision configuration (64 gas bubbles, density ratio 1000), with the
plain FP64 multigrid solver on the same system beside it, and p50/p99 of the
per-solve latency.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c3|c2|c1]

One step = one solve of the resident system from a zero initial guess.  The
inputs (1 GB per FP64 field) are far larger than the 129 MB L2, so no flush
is needed between steps.  `value` is device-timed (CUDA events on the
library's stream); `e2e` goes through the C ABI drop-in with host buffers:
the 8-coefficient Expr system (64 B/cell) copied from pinned host memory,
the solve, and the pressure copied back, every step.

N > 1 runs independent replicas (one per GPU, no collective on the data
path): every rank solves its own copy; value = all ranks' solves / max time.

--impl reference times the reference algorithm's CPU implementation on the
host cores (the C restatement of aphros's SolverConjugate in oracle/, since
the reference tree is not available where this runs) on bounded samples.
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Poisson solves/s at 1e-10 rel. residual (mixed vs FP64, same GB300); p50/p99 step latency"
UNIT = "solves/s"

WORKLOADS = {
    "c3": "mixed-precision solve, 512^3 periodic cube, 64 gas spheres r in [0.02,0.05], "
          "density ratio 1000, Taylor-Green + N(0,0.01) face noise, rel. residual 1e-10",
    "c2": "256^3 periodic cube, 16 gas spheres r in [0.03,0.08], density ratio 1000, "
          "rel. residual 1e-10",
    "c1": "64^3 periodic cube, one sphere r=0.2, density ratio 1000, rel. residual 1e-10",
}


# ---------------------------------------------------------------------------
# multi-rank helpers (replicas only)
# ---------------------------------------------------------------------------

def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def replica_share(rank, world, units):
    """Units of a job split over `world` replicas: (this rank's count,
    first unit index)."""
    base, extra = divmod(units, world)
    count = base + (1 if rank < extra else 0)
    return count, rank * base + min(rank, extra)


def aggregate_over_ranks(units, seconds):
    """(sum of units, max of seconds) over ranks (identity when not
    distributed)."""
    try:
        import torch
        import torch.distributed as dist
    except ImportError:
        return units, seconds
    if not (dist.is_available() and dist.is_initialized()):
        return units, seconds
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    s = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return int(round(u.item())), s.item()


def barrier():
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            dist.barrier()
    except ImportError:
        pass


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                     "--format=csv,noheader,nounits"],
                    capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel_name, cells):
    """DRAM bytes per launch of the kernel from the committed ncu summary
    (profiles/traffic.json: bytes per cell of one launch, measured by ncu on
    a smaller grid of the same kernel), scaled to `cells`; None if absent."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d[kernel_name]["dram_bytes_per_cell"]) * cells
    except Exception:
        return None


def rel_l2(a, b):
    a = a - a.mean()
    b = b - b.mean()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def pinned(count):
    import torch
    return torch.empty(count, dtype=torch.float64, pin_memory=True)


def cpu_baseline(case, expr8_np, threads, budget_s=15.0, cg_iters_full=None):
    """Times the oracle's CG (aphros's SolverConjugate algorithm) on the host
    cores for a bounded number of iterations; solves/s extrapolated with the
    iteration count of a full CG solve (`cg_iters_full`)."""
    import oracle
    n = case.n
    # one iteration first to size the sample
    t1 = oracle.cg_time_iters(n, expr8_np, 1, threads)
    iters = max(2, min(50, int(budget_s / max(t1, 1e-6))))
    t = oracle.cg_time_iters(n, expr8_np, iters, threads)
    per_iter = t / iters
    out = {"per_iter_s": per_iter, "iters_sampled": iters}
    if cg_iters_full:
        out["value"] = 1.0 / (per_iter * cg_iters_full)
        out["cg_iters_full"] = cg_iters_full
    return out


def cg_iterations_estimate(case_name, n_full, threads):
    """Iterations aphros's CG needs on this bubble field at ||r||/||b||=1e-10,
    measured with the CPU oracle CG on the same bubbles at n_full/8 (at
    least 32^3) and scaled by the grid ratio (CG iterations grow linearly
    with the grid edge on this operator)."""
    import oracle
    from aphros_gb300 import workload
    ns = max(32, n_full // 8)
    cs = workload.config(case_name, n=ns)
    es, _, _ = oracle.assemble_projection(ns, cs.h, cs.dt, cs.alpha, cs.rho1, cs.rho2,
                                          cs.flux)
    _, info = oracle.cg_solve(ns, cs.h, es, oracle.rel_tol(es, cs.h, 1e-10),
                              nthreads=threads)
    return int(round(info.iter * n_full / ns)), int(info.iter), ns


# algorithmic bytes per cell (compulsory traffic, each array element read or
# written once): one PLIC step = three directional sweeps, each with its
# re-reconstruction (volume fraction r/w 16, normals 24, plane constant 8,
# face flux 8, fluid flux 8, reconstruction 41), and the height curvature
# (second and fourth differences 80, heights 80, curvature with its inputs 40)
VOF_STEP_BYTES = 315
CURVATURE_BYTES = 200


def measure_vof(ctx, case, peak, peak_kind, steps, cpu=True):
    """PLIC advection + height curvature of the workload's bubble field with
    the resident corrected fluxes of the last solve: device time per step
    (CUDA events on the library stream), per-kernel bandwidth, and the
    oracle's VOF step + curvature on the host cores on a bounded sample."""
    from aphros_gb300 import _lib
    N = case.N
    ctx.flux_correct(out=False)
    ctx.vof_init(case.alpha)
    dt = case.cfl_dt(0.5)
    adv, curv, recol = [], [], []
    for s in range(steps + 2):
        ctx.vof_step(None, dt)
        a = ctx.last_timing()[0]
        ctx.curvature(out=False)
        k = ctx.last_timing()[0]
        # the connected-component colours the reference's step also computes
        ctx.vof_recolor()
        rc = ctx.last_timing()[0]
        if s >= 2:
            adv.append(a)
            curv.append(k)
            recol.append(rc)
    kernels = {}
    for kid in (_lib.K_VOF_FLUX, _lib.K_VOF_UPDATE, _lib.K_RECONSTRUCT, _lib.K_HEIGHTS,
                _lib.K_CURVATURE):
        ms_k, b_k = ctx.time_kernel(kid, reps=5)
        kernels[_lib.KERNEL_NAMES[kid]] = {"ms": round(ms_k, 4),
                                          "GB/s": round(b_k / (ms_k * 1e-3) / 1e9, 1)}
    adv_ms, curv_ms = float(np.median(adv)), float(np.median(curv))
    ach_a = VOF_STEP_BYTES * N / (adv_ms * 1e-3) / 1e9
    ach_k = CURVATURE_BYTES * N / (curv_ms * 1e-3) / 1e9
    out = {"dt_cfl": 0.5, "steps": steps,
           "advection_ms_per_step": adv_ms, "curvature_ms": curv_ms,
           "recolor_ms": float(np.median(recol)),
           "cell_steps_per_s": N / ((adv_ms + curv_ms) * 1e-3),
           "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_kind": peak_kind,
                        "advection": {"bytes_per_cell": VOF_STEP_BYTES, "achieved": ach_a,
                                      "frac": ach_a / peak},
                        "curvature": {"bytes_per_cell": CURVATURE_BYTES, "achieved": ach_k,
                                      "frac": ach_k / peak}},
           "kernels": kernels}
    if cpu:
        import oracle
        from aphros_gb300 import workload
        threads = os.cpu_count() or 1
        ns = max(32, case.n // 4)
        cs = workload.Case(ns, case.centres, case.radii, rho1=case.rho1, rho2=case.rho2,
                           seed=case.seed)
        st = oracle.VofState(ns, cs.h, cs.alpha)
        f = cs.flux
        dts = cs.cfl_dt(0.5)
        st.step(f, dts, nthreads=threads)
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            st.step(f, dts, nthreads=threads)
            st.curvature()
        per = (time.perf_counter() - t0) / reps
        out["cpu_baseline"] = {"value": ns ** 3 / per, "unit": "cell-steps/s", "cores": threads,
                               "kind": "port",
                               "sample": "%d steps of the C restatement of aphros Vof "
                                         "(Weymouth sweeps) + Heights curvature at %d^3 on "
                                         "the same bubbles and Taylor-Green flux"
                                         % (reps, ns)}
    return out


# ---------------------------------------------------------------------------
# The configuration's V-cycle: one red-black sweep before and after the
# coarse correction on the finest level, and twice as many on each coarser
# level (at most 16), the shape that is fastest at 512^3 (finest-level
# sweeps dominate the cost; coarse ones are cheap and improve the coarse
# correction).  Library defaults otherwise.
HEADLINE_MG = {"mg_pre": 1, "mg_post": 1}


def set_headline_cycle(ctx, _lib):
    ctx.set_option(_lib.OPT_CYCLE, 1)
    ctx.set_option(_lib.OPT_SWEEP_GROWTH, 3)


# arms
# ---------------------------------------------------------------------------

def run_ours(args):
    import torch
    from aphros_gb300 import _lib, workload

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local
    case = workload.config(args.workload)
    N = case.N
    ctx = _lib.Context(case.n, case.h, device)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    # the configuration's V-cycles; the W-cycle (library default at this
    # size) is measured beside them
    set_headline_cycle(ctx, _lib)
    _, bnorm = ctx.residual_norms()
    tol = 1e-10 * bnorm / math.sqrt(case.h ** 3)
    conf_mixed = _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=tol, maxiter=100, **HEADLINE_MG)
    conf_fp64 = _lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=tol, maxiter=1000, **HEADLINE_MG)

    def run_steps(conf, k, collect):
        times, launches, infos = [], 0, []
        ctx.mark(0)
        for _ in range(k):
            info = ctx.solve_resident(conf, zero_guess=True)
            ms, nl = ctx.last_timing()
            if collect:
                times.append(ms)
                launches += nl
                infos.append(info)
        ctx.mark(1)
        total_ms = ctx.elapsed(0, 1)
        return total_ms, times, launches, infos

    # warm-up (builds both hierarchies)
    for conf in (conf_mixed, conf_fp64):
        run_steps(conf, args.warmup, False)
    torch.cuda.synchronize(device)
    barrier()
    sampler = ClockSampler(device)
    with sampler:
        torch.cuda.synchronize(device)
        barrier()
        t_mixed, st_mixed, l_mixed, inf_mixed = run_steps(conf_mixed, args.steps, True)
        torch.cuda.synchronize(device)
        barrier()
    p_mixed = ctx.get_solution()
    rn, bn = ctx.residual_norms()
    rel_res_mixed = rn / bn
    t_fp64, st_fp64, l_fp64, inf_fp64 = run_steps(conf_fp64, args.steps, True)
    p_fp64 = ctx.get_solution()
    rn64, _ = ctx.residual_norms()
    units, tmax = aggregate_over_ranks(args.steps, t_mixed / 1000.0)
    units64, tmax64 = aggregate_over_ranks(args.steps, t_fp64 / 1000.0)
    value = units / tmax
    fp64_value = units64 / tmax64

    # the same solves with W-cycles below the finest level
    w_cycle = None
    if not args.no_w_cycle:
        # library defaults: W below the finest level, 2+2 sweeps on every level
        ctx.set_option(_lib.OPT_CYCLE, 0)
        ctx.set_option(_lib.OPT_SWEEP_GROWTH, 0)
        conf_mixed_w = _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=tol, maxiter=100)
        conf_fp64_w = _lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=tol, maxiter=1000)
        kw = max(1, min(args.steps, 5))
        run_steps(conf_mixed_w, 1, False)
        run_steps(conf_fp64_w, 1, False)
        tw, stw, _, infw = run_steps(conf_mixed_w, kw, True)
        rnw, bnw = ctx.residual_norms()
        pw = ctx.get_solution()
        tw64, _, _, infw64 = run_steps(conf_fp64_w, kw, True)
        set_headline_cycle(ctx, _lib)
        uw, tmw = aggregate_over_ranks(kw, tw / 1000.0)
        uw64, tmw64 = aggregate_over_ranks(kw, tw64 / 1000.0)
        w_cycle = {"value": uw / tmw, "unit": UNIT, "ms_per_step": float(tw / kw),
                   "iters": {"outer": infw[-1].iter, "inner_fp32_pcg": infw[-1].inner_iter},
                   "rel_residual": rnw / bnw, "pressure_rel_err_vs_fp64_v": rel_l2(pw, p_fp64),
                   "fp64": {"value": uw64 / tmw64, "ms_per_step": float(tw64 / kw),
                            "iters": infw64[-1].iter},
                   "mixed_over_fp64": (uw / tmw) / (uw64 / tmw64)}

    # live roofline of the dominant kernel of the mixed solve
    peak, peak_kind = measured_peak_gbs()
    kms, kbytes = ctx.time_kernel(_lib.K_SMOOTH32, reps=20)
    achieved = kbytes / (kms * 1e-3) / 1e9
    kernel_table = {}
    for kid in (_lib.K_SMOOTH32, _lib.K_APPLY32, _lib.K_RESTRICT32,
                _lib.K_APPLY64, _lib.K_SMOOTH64):
        try:
            ms_k, b_k = ctx.time_kernel(kid, reps=10)
            kernel_table[_lib.KERNEL_NAMES[kid]] = {
                "ms": round(ms_k, 4), "GB/s": round(b_k / (ms_k * 1e-3) / 1e9, 1),
                "frac": round(b_k / (ms_k * 1e-3) / 1e9 / peak, 3)}
        except _lib.AphgpuError:
            pass

    vof = None
    if not args.no_vof:
        vof = measure_vof(ctx, case, peak, peak_kind, max(3, min(args.steps, 10)),
                          cpu=(rank == 0 and not args.no_cpu))

    # end to end through the drop-in with host buffers (pinned)
    e2e = None
    if not args.no_e2e:
        expr = pinned(8 * N)
        xout = pinned(N)
        ctx._check(ctx._L.aphgpu_get_system_expr(ctx.handle, expr.data_ptr()))
        e2e_steps = max(1, min(args.steps, 5))
        info = _lib.Info()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ctx._check(ctx._L.aphgpu_set_system_expr(ctx.handle, expr.data_ptr()))
            ctx._check(ctx._L.aphgpu_solve(ctx.handle, ctypes.byref(conf_mixed), None,
                                           xout.data_ptr(), ctypes.byref(info)))
        t1 = time.perf_counter()
        eu, et = aggregate_over_ranks(e2e_steps, t1 - t0)
        e2e = {"value": eu / et, "unit": UNIT, "h2d_bytes_per_step": 8 * 8 * N,
               "d2h_bytes_per_step": 8 * N, "steps": e2e_steps,
               "path": "aphgpu_set_system_expr + aphgpu_solve (linear::Solver drop-in), "
                       "pinned host buffers"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        iters_full, iters_small, n_small = cg_iterations_estimate(args.workload, case.n, threads)
        expr_np = np.empty(8 * N)
        ctx._check(ctx._L.aphgpu_get_system_expr(ctx.handle, _lib.ptr(expr_np)))
        cb = cpu_baseline(case, expr_np, threads, budget_s=args.cpu_budget,
                          cg_iters_full=iters_full)
        cpu = {"value": cb.get("value"), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d CG iterations of the C restatement of aphros SolverConjugate "
                         "on the %d^3 system (%.3f s/iter, %d threads); full solve = %d "
                         "iterations, from the same CG on the same bubble field at "
                         "%d^3 (%d iterations) scaled by the grid ratio"
                         % (cb["iters_sampled"], case.n, cb["per_iter_s"], threads,
                            iters_full, n_small, iters_small, )}

    if rank != 0:
        return None
    lat = np.array(st_mixed)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(t_mixed / args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 multigrid in f64 defect correction (f64 residual, update, norms, coarsest solve)",
        "data": "synthetic (seeded bubble field, Taylor-Green + noise)",
        "config": {"workload": WORKLOADS[args.workload], "cells": N,
                   "grid": [case.n] * 3, "bubbles": int(len(case.radii)),
                   "density_ratio": case.rho1 / case.rho2,
                   "l2": "inputs larger than L2 (1 GB per FP64 field), no flush",
                   "multigrid": "V-cycle, red-black Gauss-Seidel 1+1 on the finest level "
                                "and 2^l+2^l (at most 16) on level l below it, coarse "
                                "couplings 60 % series + 40 % half-Galerkin; w_cycle: "
                                "library defaults (W below the finest level, 2+2 sweeps)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "fp64": {"value": fp64_value, "unit": UNIT,
                 "ms_per_step": float(t_fp64 / args.steps),
                 "p50_ms": float(np.percentile(st_fp64, 50)),
                 "p99_ms": float(np.percentile(st_fp64, 99)),
                 "iters": inf_fp64[-1].iter if inf_fp64 else None},
        "mixed_over_fp64": value / fp64_value,
        "w_cycle": w_cycle,
        "iters": {"outer": inf_mixed[-1].iter, "inner_fp32_pcg": inf_mixed[-1].inner_iter},
        "rel_residual": rel_res_mixed,
        "pressure_rel_err_vs_fp64": rel_l2(p_mixed, p_fp64),
        "cells_per_s": value * N,
        "roofline": {"bound": "hbm", "kernel": "KSmooth<float> (red-black half sweep, finest level)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": ncu_traffic("KSmooth<float>", N)},
        "kernels": kernel_table,
        "vof": vof,
        "gpu_launches": int(l_mixed),
        "e2e": e2e,
        "cpu_baseline": cpu,
        "clocks": sampler.summary(),
    }
    return line


def run_reference(args):
    """aphros's CG algorithm (oracle restatement) on the host cores."""
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    import oracle
    from aphros_gb300 import workload
    case = workload.config(args.workload)
    n, h = case.n, case.h
    threads = os.cpu_count() or 1
    e, _, _ = oracle.assemble_projection(n, h, case.dt, case.alpha, case.rho1,
                                         case.rho2, case.flux)
    # iterations of a full solve: measured on the CPU at n/8 and scaled
    iters_full, iters_small, ns = cg_iterations_estimate(args.workload, n, threads)
    per = []
    for _ in range(args.warmup):
        oracle.cg_time_iters(n, e, 1, threads)
    sample_iters = 3
    for _ in range(args.steps):
        t = oracle.cg_time_iters(n, e, sample_iters, threads)
        per.append(t / sample_iters)
    per_iter = float(np.median(per))
    value = 1.0 / (per_iter * iters_full)
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_iter * 1e3 * sample_iters,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded bubble field, Taylor-Green + noise)",
        "config": {"workload": WORKLOADS[args.workload], "cells": case.N},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "each step %d CG iterations at %d^3 (C restatement of "
                                   "aphros SolverConjugate, %d threads); full solve %d "
                                   "iterations (same CG at %d^3: %d, scaled by the grid ratio)"
                                   % (sample_iters, n, threads, iters_full, ns, iters_small)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_serve(args):
    """Served stream: Poisson-arrival step requests for resident simulations
    of edge 32-128 (log-uniform, multiples of 16, 1-8 bubbles, density ratio
    1000) on a continuous-batching server, against the same requests run one
    by one with the plain FP64 solver."""
    import random

    from aphros_gb300 import _lib, build, serve, workload
    build.build()
    cases = workload.served_cases(args.sims)
    dts = [0.5 * c.cfl_dt(0.5) for c in cases]
    rng = random.Random(5)
    order = [rng.randrange(len(cases)) for _ in range(args.requests)]

    def drive(slots, conf, rate):
        with serve.Server(budget_bytes=args.budget_gb * 1e9, slots=slots, conf=conf) as srv:
            sims = [srv.add(c, sigma=0.05) for c in cases]
            # warm-up: one step of every simulation (admission, hierarchy)
            for t in [srv.submit(sims[i], cases[i].flux, dts[i]) for i in range(len(cases))]:
                srv.wait(t)
            tickets = []
            t0 = time.perf_counter()
            clock = 0.0
            for i in order:
                if rate > 0:
                    clock += rng.expovariate(rate)
                    delay = t0 + clock - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                tickets.append(srv.submit(sims[i], cases[i].flux, dts[i]))
            res = [srv.wait(t) for t in tickets]
            t1 = time.perf_counter()
            st = srv.stats()
        lat = np.array([r.latency_ms for r in res])
        ok = all(r.status == _lib.OK and r.converged for r in res)
        return {"steps_per_s": len(res) / (t1 - t0), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "all_converged": ok,
                "evictions": int(st.evictions), "resident_gb": st.resident_bytes / 1e9}

    mixed = _lib.default_conf(solver=_lib.SOLVER_MIXED, rtol=1e-10)
    plain = _lib.default_conf(solver=_lib.SOLVER_MGPCG, rtol=1e-10)
    one_by_one = drive(1, plain, 0.0)
    saturated = drive(args.slots, mixed, 0.0)
    rates = {}
    for rate in args.rates:
        rates[str(rate)] = drive(args.slots, mixed, rate)
    cells = [c.N for c in cases]
    return {
        "metric": "served steps/s and p50/p99 step latency (projection + PLIC advection + "
                  "curvature per step)",
        "value": saturated["steps_per_s"], "unit": "steps/s", "n_gpus": 1,
        "higher_is_better": True,
        "config": {"workload": "served stream, %d resident simulations of edge 32-128 "
                               "(log-uniform, multiples of 16), 1-8 bubbles, density ratio "
                               "1000, %d requests, %d slots, %g GB budget"
                               % (len(cases), args.requests, args.slots, args.budget_gb),
                   "cells_mean": float(np.mean(cells))},
        "served_saturated": saturated, "served_at_rate": rates,
        "one_by_one_plain_fp64": one_by_one,
        "speedup_vs_one_by_one": saturated["steps_per_s"] / one_by_one["steps_per_s"],
    }


def run_batch(args):
    """Batched configuration: `--domains` independent periodic domains of
    edge {32,48,64,96} (1-8 bubbles, density ratio log-uniform in
    [10,1000]), all solved to ||r||/||b|| = 1e-10 by the batched
    mixed-precision solver (one launch per multigrid level for every domain,
    inner iterations replayed from a CUDA graph, autotuned tiles and sweeps),
    against the same domains solved one after another by the per-domain
    mixed and plain FP64 multigrid solvers."""
    import torch

    from aphros_gb300 import _lib, build, workload
    build.build()
    cases = workload.batch_cases(args.domains)
    maxn = max(c.N for c in cases)
    pa, pf = pinned(maxn).numpy(), pinned(3 * maxn).numpy()
    ctxs = []
    t0 = time.perf_counter()
    for c in cases:
        ctx = _lib.Context(c.n, c.h, 0)
        a, f = pa[:c.N], pf[:3 * c.N]
        a[:] = c.alpha
        f[:] = c.flux
        ctx.assemble_projection(a, c.rho1, c.rho2, f, c.dt)
        c._alpha = c._flux = None
        ctxs.append(ctx)
    setup_s = time.perf_counter() - t0
    cells = sum(c.N for c in cases)
    conf = _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=0.0, rtol=1e-10)
    batch = _lib.Batch(ctxs)
    t0 = time.perf_counter()
    if args.tiles:
        batch.set_tiles(*args.tiles)
        tuned_ms = None
    else:
        tuned_ms = batch.tune(conf)
    tune_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        infos = batch.solve(conf)
    dev_ms, wall_ms = [], []
    launches0 = batch.last()[1]
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            infos = batch.solve(conf)
            wall_ms.append(1e3 * (time.perf_counter() - w0))
            dev_ms.append(batch.last()[0])
    launches = (batch.last()[1] - launches0) / args.steps
    conv = all(i.converged for i in infos)
    worst = max(ctx.residual_norms()[0] / ctx.residual_norms()[1] for ctx in ctxs)
    x_batch = [ctx.get_solution() for ctx in ctxs]

    def one_by_one(solver):
        cf = _lib.default_conf(solver=solver, tol=0.0, rtol=1e-10)
        for ctx in ctxs:  # warm pass (hierarchies, graphs)
            ctx.solve_resident(cf, zero_guess=True)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        its = []
        for ctx in ctxs:
            its.append(ctx.solve_resident(cf, zero_guess=True).iter)
        return 1e3 * (time.perf_counter() - w0), its

    mixed_ms, _ = one_by_one(_lib.SOLVER_MIXED)
    dev = [rel_l2(x_batch[q], ctxs[q].get_solution()) for q in range(len(ctxs))]
    fp64_ms, _ = one_by_one(_lib.SOLVER_MGPCG)
    # end to end through the C ABI: every domain's 8-coefficient system from
    # pinned host memory, the batched solve, every pressure back
    e2e_ms = None
    if not args.no_e2e:
        pe = pinned(8 * maxn).numpy()
        px = pinned(maxn).numpy()
        host = [ctx.get_system_expr() for ctx in ctxs]
        t_e = []
        for rep in range(2):
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            for ctx, e in zip(ctxs, host):
                pe[:e.size] = e
                ctx.set_system_expr(pe[:e.size])
            infos_e = batch.solve(conf)
            for ctx in ctxs:
                ctx._check(ctx._L.aphgpu_get_solution(ctx.handle, _lib.ptr(px[:ctx.N])))
            t_e.append(1e3 * (time.perf_counter() - w0))
        e2e_ms = t_e[-1]
        conv = conv and all(i.converged for i in infos_e)
    ms = float(np.median(dev_ms))
    n = len(cases)
    line = {
        "metric": "batched domain solves/s at 1e-10 rel. residual (mixed precision)",
        "value": n / (ms / 1e3), "unit": "domain solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded spheres, Taylor-Green + noise)",
        "config": {"workload": "batched: %d periodic domains, edge in {32,48,64,96}, 1-8 "
                               "bubbles, density ratio log-uniform [10,1000], %d cells total; "
                               "inputs %.1f GB > L2, no flush" % (n, cells, cells * 40 / 1e9),
                   "tuned": {"mg_sweeps": conf.mg_pre, "tile_planes": batch.tiles()[0],
                             "coarse_cycle": "W" if batch.cycle() == 2 else "V",
                             "coarse_cells": batch.tiles()[1], "tune_s": tune_s,
                             "best_tune_ms": tuned_ms}},
        "wall_ms_per_step": float(np.median(wall_ms)),
        "gpu_launches": launches,
        "all_converged": conv, "worst_rel_residual": worst,
        "outer_iters_mean": float(np.mean([i.iter for i in infos])),
        "inner_iters_mean": float(np.mean([i.inner_iter for i in infos])),
        "inner_iters_max": int(max(i.inner_iter for i in infos)),
        "max_rel_l2_vs_per_domain_mixed": max(dev),
        "one_by_one_mixed_ms": mixed_ms, "one_by_one_fp64_ms": fp64_ms,
        "speedup_vs_one_by_one_mixed": mixed_ms / ms,
        "speedup_vs_one_by_one_fp64": fp64_ms / ms,
        "setup_s": setup_s,
        "clocks": clk.summary(),
    }
    if e2e_ms is not None:
        line["e2e"] = {"value": n / (e2e_ms / 1e3), "unit": "domain solves/s",
                       "h2d_bytes_per_step": 64 * cells, "d2h_bytes_per_step": 8 * cells}
    batch.close()
    return line


def run_profile(args):
    """Solves only (for ncu launch lists and captures)."""
    from aphros_gb300 import _lib, build, workload
    build.build()
    if args.profile == "batch":
        ctxs = []
        for c in workload.batch_cases(args.domains):
            ctx = _lib.Context(c.n, c.h, 0)
            ctx.assemble_projection(c.alpha, c.rho1, c.rho2, c.flux, c.dt)
            ctxs.append(ctx)
        batch = _lib.Batch(ctxs)
        if args.tiles:
            batch.set_tiles(*args.tiles)
        if args.cycle in (1, 2):
            batch.set_cycle(args.cycle)
        conf = _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=0.0, rtol=1e-10)
        l0 = 0
        for s in range(args.warmup + args.steps):
            if s == args.warmup:
                l0 = batch.last()[1]
            infos = batch.solve(conf)
        print("profile batch: %d domains, %.3f ms last solve, %d launches per solve, "
              "inner iterations max %d" % (len(ctxs), batch.last()[0],
                                           (batch.last()[1] - l0) // max(args.steps, 1),
                                           max(i.inner_iter for i in infos)))
        return
    case = workload.config(args.workload)
    ctx = _lib.Context(case.n, case.h, 0)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    _, bnorm = ctx.residual_norms()
    tol = 1e-10 * bnorm / math.sqrt(case.h ** 3)
    solver = _lib.SOLVER_MGPCG if args.profile == "fp64" else _lib.SOLVER_MIXED
    if args.cycle == 1:
        # the configuration's V-cycle (as in the headline)
        set_headline_cycle(ctx, _lib)
        conf = _lib.default_conf(solver=solver, tol=tol, **HEADLINE_MG)
    else:
        ctx.set_option(_lib.OPT_CYCLE, args.cycle)
        conf = _lib.default_conf(solver=solver, tol=tol)
    if args.profile == "vof":
        # one solve, the corrected fluxes, then `warmup` + `steps` PLIC steps
        # with the height curvature after each
        ctx.solve_resident(conf, zero_guess=True)
        ctx.flux_correct(out=False)
        ctx.vof_init(case.alpha)
        dt = case.cfl_dt(0.5)
        for _ in range(args.warmup + args.steps):
            ctx.vof_step(None, dt)
            ctx.curvature(out=False)
        print("profile vof: %d steps of %d^3" % (args.warmup + args.steps, case.n))
        return
    for _ in range(args.warmup + args.steps):
        info = ctx.solve_resident(conf, zero_guess=True)
    print("profile %s: %d iterations (%d inner), %d launches in the last solve"
          % (args.profile, info.iter, info.inner_iter, ctx.last_timing()[1]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c3")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-w-cycle", action="store_true",
                    help="skip the W-cycle measurement beside the V-cycle headline")
    ap.add_argument("--no-vof", action="store_true",
                    help="skip the PLIC advection + curvature measurement")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--cycle", type=int, choices=[0, 1, 2], default=0,
                    help="--profile: 1 the headline's V-cycle configuration, 2 W, 0 "
                         "library default (batch: the per-domain coarse cycle)")
    ap.add_argument("--profile", choices=["mixed", "fp64", "batch", "vof"], default=None,
                    help="profiling run: assemble, then `steps` solves of one solver "
                         "after `warmup` solves, no other work and no output line")
    ap.add_argument("--serve", action="store_true",
                    help="served-stream benchmark instead of the solve benchmark")
    ap.add_argument("--sims", type=int, default=64)
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--rates", type=float, nargs="*", default=[50.0, 200.0])
    ap.add_argument("--batch", action="store_true",
                    help="batched-domains benchmark instead of the solve benchmark")
    ap.add_argument("--domains", type=int, default=512)
    ap.add_argument("--tiles", type=int, nargs=2, default=None,
                    metavar=("PLANES", "COARSE_CELLS"),
                    help="batched tiling instead of the autotuner")
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.serve:
        print(json.dumps(run_serve(args)), flush=True)
        return
    if args.batch:
        args.warmup = max(args.warmup, 3)
        print(json.dumps(run_batch(args)), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        line = run_reference(args)
    else:
        from aphros_gb300 import build
        build.build()
        line = run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
