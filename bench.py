"""Benchmark of the projection-step pressure solve on GB300.

Headline metric: Poisson solves/s at ||r||/||b|| = 1e-10 on the 512^3
mixed-precision configuration (64 gas bubbles, density ratio 1000), with the
plain FP64 multigrid solver on the same system beside it, p50/p99 of the
per-solve latency, and every pressure's relative L2 distance to a tight FP64
solution (MG-PCG to ||r||/||b|| = 1e-13; the bar is 1e-9).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c3|c2|c1]

One step = one solve of the resident system from a zero initial guess.  The
inputs (1 GB per FP64 field) are far larger than the 129 MB L2, so no flush
is needed between steps.  `value` is device-timed (CUDA events on the
library's stream); `e2e` goes through the C ABI drop-in with host buffers:
the 8-coefficient Expr system (64 B/cell) copied from pinned host memory,
the solve, and the pressure copied back, every step.

The headline runs the library defaults (W-cycle below the finest level, 2+2
red-black sweeps).  The same line carries the other configurations (one
GPU): the literal C3 cycle (V, 2+2 sweeps) and the fastest V-cycle beside
the headline; `c2_pipeline`
(256^3, 100 steps of solve + PLIC advection + curvature); `c4_batch` (512
uneven domains in one batched solve); `c5_serve` (2000 resident simulations,
Poisson arrivals at 50-2000 steps/s under a 150 GB budget).

N > 1 runs independent replicas (one per GPU, no collective on the data
path): every rank solves its own copy; value = all ranks' solves / max time.

--impl reference times the reference's CPU solve on the host cores: aphros's
own SolverConjugate compiled from its sources (oracle/ref) where they are
staged, else the C restatement of it in oracle/, on bounded samples.
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


def cg_iterations_full(case_name, n_full, threads):
    """Iterations aphros's CG needs at ||r||/||b|| = 1e-10 on this bubble
    field at n_full^3: the fit iters = a * n^b of the counts the oracle CG
    (the algorithm of SolverConjugate) measured at 64^3, 128^3 and 256^3
    (oracle/data/cg_iterations.json, made by make_cg_iterations.py there).
    Without that file: measured at n_full/8 and scaled by the grid ratio."""
    p = os.path.join(ROOT, "oracle", "data", "cg_iterations.json")
    if case_name == "c3":
        try:
            with open(p) as f:
                d = json.load(f)
            a, b = d["fit"]["a"], d["fit"]["b"]
            rows = ", ".join("%d^3: %d" % (r["n"], r["iters"]) for r in d["rows"])
            return int(round(a * n_full ** b)), ("fit %.3g * n^%.3f of the oracle CG's counts "
                                                 "(%s)" % (a, b, rows))
        except (OSError, KeyError, ValueError):
            pass
    import oracle
    from aphros_gb300 import workload
    ns = max(32, n_full // 8)
    cs = workload.config(case_name, n=ns)
    es, _, _ = oracle.assemble_projection(ns, cs.h, cs.dt, cs.alpha, cs.rho1, cs.rho2,
                                          cs.flux)
    _, info = oracle.cg_solve(ns, cs.h, es, oracle.rel_tol(es, cs.h, 1e-10),
                              nthreads=threads)
    return (int(round(info.iter * n_full / ns)),
            "oracle CG at %d^3 (%d iterations) scaled by the grid ratio" % (ns, info.iter))


def cpu_model():
    """CPU model of the host, from /proc/cpuinfo (or the platform string)."""
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        for key in ("model name", "Model Name", "CPU part"):
            for line in txt.splitlines():
                if line.lower().startswith(key.lower()):
                    val = line.split(":", 1)[1].strip()
                    if key == "CPU part":
                        imp = [ln.split(":", 1)[1].strip() for ln in txt.splitlines()
                               if ln.lower().startswith("cpu implementer")]
                        return "arm implementer %s part %s" % (imp[0] if imp else "?", val)
                    return val
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


REF_HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def reference_cg_seconds(case, iters, threads, blocks=32):
    """aphros's own SolverConjugate (compiled from the reference sources by
    oracle/ref/Makefile into ref_harness) on the workload's projection
    system, assembled by aphros's Proj code from the same volume fraction
    and fluxes: exactly `iters` CG iterations on `threads` OpenMP threads,
    blocks of blocks^3 cells.  Returns (seconds per iteration, iterations,
    harness wall seconds) or None when the harness is not built."""
    import tempfile
    if not os.access(REF_HARNESS, os.X_OK):
        return None
    with tempfile.TemporaryDirectory() as tmp:
        case.alpha.tofile(os.path.join(tmp, "a.bin"))
        case.flux.tofile(os.path.join(tmp, "f.bin"))
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        bs = min(blocks, case.n)
        t0 = time.perf_counter()
        r = subprocess.run([REF_HARNESS, "cgtime", str(case.n), str(bs), repr(case.dt),
                            repr(case.rho1), repr(case.rho2), str(iters), "a.bin", "f.bin",
                            "cg"], cwd=tmp, env=env, stdout=subprocess.PIPE,
                           stderr=subprocess.STDOUT, text=True)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            print("reference harness failed: %s" % r.stdout[-500:], file=sys.stderr)
            return None
        with open(os.path.join(tmp, "cg.time")) as f:
            sec, it = f.read().split()[:2]
    it = int(it)
    return float(sec) / max(it, 1), it, wall


def cpu_baseline(case, case_name, threads, budget_s=15.0, expr8_np=None):
    """The reference's CPU CG on the host cores, on a bounded sample: aphros's
    own SolverConjugate through ref_harness when built ("reference"), else
    the oracle's C restatement ("port").  Solves/s from the time per
    iteration and the iteration count of a full solve."""
    iters_full, how = cg_iterations_full(case_name, case.n, threads)
    # a sample of about budget_s of CG iterations (rate of the port first)
    out = None
    ref = reference_cg_seconds(case, max(2, int(budget_s / 1.0)), threads)
    if ref is not None:
        per_iter, it, wall = ref
        out = {"kind": "reference", "per_iter_s": per_iter, "iters_sampled": it,
               "sample": "%d iterations of aphros's own SolverConjugate (compiled from its "
                         "sources, blocks of 32^3, %d OpenMP threads) on the %d^3 system "
                         "assembled by aphros's Proj code (%.3f s/iteration; %.0f s with "
                         "the assembly); full solve = %d iterations (%s)"
                         % (it, threads, case.n, per_iter, wall, iters_full, how)}
    else:
        import oracle
        if expr8_np is None:
            expr8_np, _, _ = oracle.assemble_projection(case.n, case.h, case.dt, case.alpha,
                                                        case.rho1, case.rho2, case.flux)
        t1 = oracle.cg_time_iters(case.n, expr8_np, 1, threads)
        iters = max(2, min(50, int(budget_s / max(t1, 1e-6))))
        per_iter = oracle.cg_time_iters(case.n, expr8_np, iters, threads) / iters
        out = {"kind": "port", "per_iter_s": per_iter, "iters_sampled": iters,
               "sample": "%d CG iterations of the C restatement of aphros SolverConjugate on "
                         "the %d^3 system (%.3f s/iter, %d threads); full solve = %d "
                         "iterations (%s)" % (iters, case.n, per_iter, threads, iters_full,
                                              how)}
    out.update({"value": 1.0 / (out["per_iter_s"] * iters_full), "unit": UNIT,
                "cores": threads, "cpu": cpu_model(), "cg_iters_full": iters_full})
    return out


# algorithmic bytes per cell of the dense formulation (each array element
# read or written once): one PLIC step = three directional sweeps, each
# with its re-reconstruction (volume fraction r/w 16, normals 24, plane
# constant 8, face flux 8, fluid flux 8, reconstruction 41), and the height
# curvature (second and fourth differences 80, heights 80, curvature with
# its inputs 40)
VOF_STEP_BYTES = 315
CURVATURE_BYTES = 200
# the device path touches normals, plane constants, fluid fluxes and
# heights of interfacial cells only: its compulsory traffic per step is
# three fused directional passes (u read and written, face flux, fcuu:
# 25 B/cell each; the last one also writes the next step's fcuu, 1 B/cell,
# so a step that follows a step needs no interface listing) and, per
# interfacial cell, about 112 B per direction (flux through its
# faces: normal, plane constant, u, two face fluxes and fluid fluxes;
# re-reconstruction: u, normal and plane constant written); the curvature
# writes kappa for every cell (8 B/cell) and reads/writes about 88 B per
# interfacial cell (u, normal, three heights written and read, kappa)
VOF_DEVICE_BYTES_CELL = 3 * 25 + 1
VOF_DEVICE_BYTES_IF = 3 * 112
CURV_DEVICE_BYTES_CELL = 8
CURV_DEVICE_BYTES_IF = 88


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
    # the particle-string and hybrid estimators on the last state (the
    # reference's default estimator is particles)
    part, hyb = [], []
    for _ in range(3):
        ctx.curvature_estimator(_lib.CURV_PARTICLES, out=False)
        part.append(ctx.last_timing()[0])
        ctx.curvature_estimator(_lib.CURV_HYBRID, out=False)
        hyb.append(ctx.last_timing()[0])
    ctx.curvature(out=False)
    adv_ms, curv_ms = float(np.median(adv)), float(np.median(curv))
    ach_a = VOF_STEP_BYTES * N / (adv_ms * 1e-3) / 1e9
    # interfacial cells of the last step (u alone read back)
    u = np.empty(N)
    ctx._check(ctx._L.aphgpu_vof_get(ctx._p, _lib.ptr(u), None, None, None))
    nif = int(np.count_nonzero((u > 0) & (u < 1)))
    del u
    dev_a = VOF_DEVICE_BYTES_CELL * N + VOF_DEVICE_BYTES_IF * nif
    dev_k = CURV_DEVICE_BYTES_CELL * N + CURV_DEVICE_BYTES_IF * nif
    ach_da = dev_a / (adv_ms * 1e-3) / 1e9
    ach_dk = dev_k / (curv_ms * 1e-3) / 1e9
    out = {"dt_cfl": 0.5, "steps": steps,
           "advection_ms_per_step": adv_ms, "curvature_ms": curv_ms,
           "recolor_ms": float(np.median(recol)),
           "cell_steps_per_s": N / ((adv_ms + curv_ms) * 1e-3),
           "interfacial_cells": nif,
           "curvature_particles_ms": float(np.median(part)),
           "curvature_hybrid_ms": float(np.median(hyb)),
           "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_kind": peak_kind,
                        "advection": {"bytes_per_cell": VOF_STEP_BYTES, "achieved": ach_a,
                                      "frac": ach_a / peak,
                                      "device_bytes_per_cell": dev_a / N,
                                      "device_achieved": ach_da,
                                      "device_frac": ach_da / peak},
                        "curvature": {"bytes_per_cell": dev_k / N, "achieved": ach_dk,
                                      "frac": ach_dk / peak,
                                      "dense_bytes_per_cell": CURVATURE_BYTES,
                                      "note": "bytes of the interface-list algorithm: kappa "
                                              "of every cell, heights and inputs of "
                                              "interfacial cells; the dense formulation's "
                                              "200 B/cell are not moved"}},
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
        # the particle estimator of the reference, restated (the oracle),
        # on the same sample state with all host threads
        t0 = time.perf_counter()
        kp = oracle.curv_particles(ns, cs.h, st.u, st.nrm, st.a, nthreads=threads)
        part_s = time.perf_counter() - t0
        nifs = int(np.count_nonzero(~np.isnan(kp)))
        out["cpu_particles"] = {"interfacial_cells_per_s": nifs / part_s, "cores": threads,
                                "kind": "port",
                                "sample": "curvature::Particles (part_* defaults) restated "
                                          "in C, %d interfacial cells of the %d^3 sample "
                                          "state, %.3f s" % (nifs, ns, part_s)}
        out["gpu_particles_interfacial_cells_per_s"] = nif / (out["curvature_particles_ms"]
                                                              * 1e-3)
        out["cpu_baseline"] = {"value": ns ** 3 / per, "unit": "cell-steps/s", "cores": threads,
                               "kind": "port",
                               "sample": "%d steps of the C restatement of aphros Vof "
                                         "(Weymouth sweeps) + Heights curvature at %d^3 on "
                                         "the same bubbles and Taylor-Green flux"
                                         % (reps, ns)}
    return out


# ---------------------------------------------------------------------------
# The headline solve runs the library defaults: a W-cycle below the finest
# level from 256^3 cells up (its levels of at most 16^3 cells visiting the
# level below once), 2 pre- and 2 post-smoothing red-black sweeps
# on every level (the levels of at most 8^3 cells cycled by one CTA per
# visit, the finest FP32 level in the colour-split order), inner FP32 PCG
# to 3e-4, the outer residual after the first updated in double-float
# arithmetic, stopped at ||r||/||b|| <= 1e-10.  Measured at 512^3 it is the
# fastest configuration whose pressure is within the 1e-9 bar of a tight
# FP64 solution (4.9e-10) at that stop.  The
# configuration's literal cycle (V, 2+2 sweeps on every level) and the
# fastest V-cycle (one sweep before and after on the finest level, 2^l on
# level l below it, inner PCG to 1e-3, which keeps its pressure within the
# bar at 1e-10) are measured beside it.  The FP64 comparator runs the same
# defaults (also its fastest configuration: 489 ms against 637 ms for the
# V-cycle shape).
HEADLINE_MG = {}
HEADLINE_STOP = 1e-10
V_CYCLE_MG = {"mg_pre": 1, "mg_post": 1, "inner_rtol": 1e-3}
PRESSURE_BAR = 1e-9
# algorithmic bytes per cell of one FP32 red-black sweep (both colours): x
# read 4 + x written 4 + b 4 + couplings 12 = 24 (the FP64 48 halved); a
# half sweep (one colour) is half of that
SWEEP_BYTES = 24.0
HALF_SWEEP_BYTES = 12.0


def color_split_used(shape):
    """Whether the mixed solver keeps its finest FP32 level in the
    colour-split order (the library default, taken from 2^22 cells up when
    nx % 8 == 0 and ny, nz are even): the half sweep then moves 18 of the 24
    bytes per cell of the natural order's."""
    nx, ny, nz = (shape,) * 3 if isinstance(shape, int) else shape
    return (nx % 8 == 0 and nx >= 16 and ny % 2 == 0 and nz % 2 == 0 and
            nx * ny * nz >= 1 << 22)


def set_v_cycle(ctx, _lib):
    ctx.set_option(_lib.OPT_CYCLE, 1)
    ctx.set_option(_lib.OPT_SWEEP_GROWTH, 3)


def set_headline_cycle(ctx, _lib):
    set_default_cycle(ctx, _lib)


def set_literal_cycle(ctx, _lib):
    ctx.set_option(_lib.OPT_CYCLE, 1)
    ctx.set_option(_lib.OPT_SWEEP_GROWTH, 1)


def set_default_cycle(ctx, _lib):
    ctx.set_option(_lib.OPT_CYCLE, 0)
    ctx.set_option(_lib.OPT_SWEEP_GROWTH, 0)


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
    _, bnorm = ctx.residual_norms()
    abs_tol = lambda rt: rt * bnorm / math.sqrt(case.h ** 3)
    tol = abs_tol(1e-10)

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

    # the tight FP64 reference of the pressure bar: MG-PCG (W-cycle) to
    # ||r||/||b|| = 1e-13, untimed
    set_default_cycle(ctx, _lib)
    ctx.set_option(_lib.OPT_CYCLE, 2)
    ctx.solve_resident(_lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=abs_tol(1e-13),
                                         maxiter=1000), zero_guess=True)
    rn_t, bn_t = ctx.residual_norms()
    p_tight = ctx.get_solution()
    set_headline_cycle(ctx, _lib)

    conf_mixed = _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=abs_tol(HEADLINE_STOP),
                                   maxiter=100, **HEADLINE_MG)
    conf_fp64 = _lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=tol, maxiter=1000, **HEADLINE_MG)
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
    err_mixed = rel_l2(p_mixed, p_tight)
    err_fp64 = rel_l2(p_fp64, p_tight)
    def variant(setter, mg, k):
        setter(ctx, _lib)
        cm = _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=tol, maxiter=100, **mg)
        mg64 = {key: v for key, v in mg.items() if not key.startswith("inner")}
        cf = _lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=tol, maxiter=1000, **mg64)
        run_steps(cm, 1, False)
        run_steps(cf, 1, False)
        tm, _, _, im = run_steps(cm, k, True)
        rnm, bnm = ctx.residual_norms()
        pm = ctx.get_solution()
        tf, _, _, iff = run_steps(cf, k, True)
        pf = ctx.get_solution()
        um, tmm = aggregate_over_ranks(k, tm / 1000.0)
        uf, tmf = aggregate_over_ranks(k, tf / 1000.0)
        set_headline_cycle(ctx, _lib)
        em, ef = rel_l2(pm, p_tight), rel_l2(pf, p_tight)
        return {"value": um / tmm, "unit": UNIT, "ms_per_step": float(tm / k),
                "iters": {"outer": im[-1].iter, "inner_fp32_pcg": im[-1].inner_iter},
                "rel_residual": rnm / bnm, "pressure_rel_err_vs_tight_fp64": em,
                "fp64": {"value": uf / tmf, "ms_per_step": float(tf / k),
                         "iters": iff[-1].iter, "pressure_rel_err_vs_tight_fp64": ef},
                "mixed_over_fp64": (um / tmm) / (uf / tmf),
                "within_bar": bool(em <= PRESSURE_BAR and ef <= PRESSURE_BAR)}

    kv = max(1, min(args.steps, 3))
    # the configuration's literal cycle: V, 2+2 red-black sweeps on every level
    literal = variant(set_literal_cycle, {"mg_pre": 2, "mg_post": 2}, kv)
    # the fastest V-cycle: 1+1 on the finest level, 2^l+2^l below
    v_cycle = None if args.no_v_cycle else variant(set_v_cycle, V_CYCLE_MG, kv)

    # live roofline of the dominant kernel of the mixed solve: the fused
    # red-black sweep of the finest level (the smoother), else the half
    # sweep when the fused one is off
    peak, peak_kind = measured_peak_gbs()
    try:
        kms, _ = ctx.time_kernel(_lib.K_SWEEP32, reps=20)
        kname, kbytes = "KSweepPipe (fused red-black sweep, finest level)", SWEEP_BYTES * N
        traffic = ncu_traffic("KSweepPipe", N)
    except _lib.AphgpuError:
        kms, _ = ctx.time_kernel(_lib.K_SMOOTH32, reps=20)
        if color_split_used(case.n):
            kname = "KSmoothSplit (colour-split red-black half sweep, finest level)"
            traffic = ncu_traffic("KSmoothSplit", N)
        else:
            kname = "KSmooth<float> (red-black half sweep, finest level)"
            traffic = ncu_traffic("KSmooth<float>", N)
        kbytes = HALF_SWEEP_BYTES * N
    achieved = kbytes / (kms * 1e-3) / 1e9
    kernel_table = {}
    for kid in (_lib.K_SMOOTH32, _lib.K_SWEEP32, _lib.K_APPLY32, _lib.K_RESTRICT32,
                _lib.K_APPLY64, _lib.K_SMOOTH64):
        try:
            ms_k, b_k = ctx.time_kernel(kid, reps=10)
            kernel_table[_lib.KERNEL_NAMES[kid]] = {
                "ms": round(ms_k, 4), "GB/s": round(b_k / (ms_k * 1e-3) / 1e9, 1),
                "frac": round(b_k / (ms_k * 1e-3) / 1e9 / peak, 3)}
        except _lib.AphgpuError:
            pass
    # the fused full sweeps (one launch per red-black sweep, 24 B/cell) beside
    # the half sweeps above; the solve keeps the half sweeps, which are faster
    # on this part, and these two entries show by how much
    for mode, label in ((1, "KSweepPipe (fused sweep, option 1)"),
                        (5, "KSweepWave (in-place wavefront sweep, option 5)")):
        try:
            ctx.set_option(_lib.OPT_FUSED_SWEEPS, mode)
            run_steps(conf_mixed, 1, False)
            ms_k, b_k = ctx.time_kernel(_lib.K_SWEEP32, reps=10)
            kernel_table[label] = {
                "ms": round(ms_k, 4), "GB/s": round(b_k / (ms_k * 1e-3) / 1e9, 1),
                "frac": round(b_k / (ms_k * 1e-3) / 1e9 / peak, 3)}
        except _lib.AphgpuError:
            pass
    ctx.set_option(_lib.OPT_FUSED_SWEEPS, 0)
    run_steps(conf_mixed, 1, False)  # rebuilds the levels for the e2e arm

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
    ctx.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cpu = cpu_baseline(case, args.workload, threads, budget_s=args.cpu_budget)

    # the other configurations, on one GPU only
    subs = {}
    if world == 1 and args.workload == "c3":
        if not args.no_pipeline:
            subs["c2_pipeline"] = measure_pipeline(args)
        if not args.no_batch:
            sub = argparse.Namespace(**vars(args))
            sub.steps, sub.warmup = max(2, min(args.steps, 5)), 2
            subs["c4_batch"] = run_batch(sub)
        if not args.no_serve:
            sub = argparse.Namespace(**vars(args))
            sub.sims, sub.requests = args.serve_sims, args.serve_requests
            sub.rates = args.serve_rates
            subs["c5_serve"] = run_serve(sub)

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
                   "multigrid": "library defaults: W-cycle below the finest level, "
                                "red-black Gauss-Seidel 2+2 on every level (levels of at "
                                "most 8^3 cells cycled by one CTA per visit), coarse "
                                "couplings 60 % series + 40 % half-Galerkin, inner FP32 PCG "
                                "to 3e-4; "
                                "literal_c3_cycle: V, 2+2 on every level; v_cycle: V, 1+1 on "
                                "the finest level and 2^l+2^l (at most 16) on level l below "
                                "it, inner PCG to 1e-3",
                   "stop": "||r||/||b|| <= %g (mixed and FP64)" % HEADLINE_STOP,
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "fp64": {"value": fp64_value, "unit": UNIT,
                 "ms_per_step": float(t_fp64 / args.steps),
                 "p50_ms": float(np.percentile(st_fp64, 50)),
                 "p99_ms": float(np.percentile(st_fp64, 99)),
                 "iters": inf_fp64[-1].iter if inf_fp64 else None,
                 "pressure_rel_err_vs_tight_fp64": err_fp64},
        "mixed_over_fp64": value / fp64_value,
        "pressure_rel_err_vs_tight_fp64": err_mixed,
        "pressure_rel_err_vs_fp64_solve": rel_l2(p_mixed, p_fp64),
        "tight_fp64_rel_residual": rn_t / bn_t,
        "within_1e-9": bool(err_mixed <= PRESSURE_BAR and err_fp64 <= PRESSURE_BAR),
        "literal_c3_cycle": literal,
        "v_cycle": v_cycle,
        "iters": {"outer": inf_mixed[-1].iter, "inner_fp32_pcg": inf_mixed[-1].inner_iter},
        "rel_residual": rel_res_mixed,
        "cells_per_s": value * N,
        "roofline": {"bound": "hbm",
                     "kernel": kname, "ms": kms,
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes": kbytes, "traffic": traffic,
                     "traffic_over_algorithmic": (traffic / kbytes) if traffic else None},
        "kernels": kernel_table,
        "vof": vof,
        "gpu_launches": int(l_mixed),
        "e2e": e2e,
        "cpu_baseline": cpu,
        "clocks": sampler.summary(),
    }
    line.update(subs)
    return line


def measure_pipeline(args, steps=100):
    """C2: 256^3, 16 bubbles, density ratio 1000; `steps` time steps of the
    projection (assembly from the resident volume fraction and the predicted
    fluxes, mixed solve to 1e-10 warm-started from the resident pressure,
    flux correction) + PLIC advection + height curvature, everything
    resident on the device; against the same steps with the FP64 MG-PCG."""
    import torch
    from aphros_gb300 import _lib, workload
    case = workload.config("c2")
    dt = case.cfl_dt(0.5)
    flux = pinned(3 * case.N).numpy()
    flux[:] = case.flux
    out = {"workload": "C2: 256^3 periodic cube, 16 gas spheres r in [0.03,0.08], density "
                       "ratio 1000, Taylor-Green + N(0,0.01) predicted fluxes, %d steps of "
                       "solve (rel. residual 1e-10, warm start) + PLIC advection (CFL 0.5) "
                       "+ height curvature" % steps}
    for name, solver in (("mixed", _lib.SOLVER_MIXED), ("fp64", _lib.SOLVER_MGPCG)):
        ctx = _lib.Context(case.n, case.h, 0)
        ctx.vof_init(case.alpha)
        conf = _lib.default_conf(solver=solver, tol=0.0, rtol=1e-10, maxiter=1000)
        dev = {"solve": 0.0, "vof": 0.0, "curvature": 0.0}
        iters, vol0 = [], None
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for s in range(steps):
            ctx._check(ctx._L.aphgpu_assemble_projection(ctx.handle, None, case.rho1, case.rho2,
                                                         _lib.ptr(flux), None, case.dt, 1))
            info = ctx.solve_resident(conf, zero_guess=(s == 0))
            dev["solve"] += ctx.last_timing()[0]
            iters.append(info.iter if solver == _lib.SOLVER_MGPCG else info.inner_iter)
            ctx.flux_correct(out=False)
            ctx.vof_step(None, dt)
            dev["vof"] += ctx.last_timing()[0]
            ctx.curvature(out=False)
            dev["curvature"] += ctx.last_timing()[0]
            if s == 0:
                vol0 = float(ctx.vof_get()[0].sum())
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        vol1 = float(ctx.vof_get()[0].sum())
        out[name] = {"steps_per_s": steps / wall, "wall_ms_per_step": 1e3 * wall / steps,
                     "device_ms_per_step": {k: v / steps for k, v in dev.items()},
                     "iters_mean": float(np.mean(iters)), "iters_first": iters[0],
                     "volume_drift_rel": abs(vol1 - vol0) / vol0}
        ctx.close()
    out["mixed_over_fp64"] = out["mixed"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    return out


def run_reference(args):
    """The reference's CPU solve on the host cores: aphros's own
    SolverConjugate compiled from its sources (ref_harness), else the
    oracle's C restatement.  Each step is one CG iteration of the workload's
    system; solves/s = 1 / (seconds per iteration x iterations of a full
    solve)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    import oracle
    from aphros_gb300 import workload
    case = workload.config(args.workload)
    n, h = case.n, case.h
    threads = os.cpu_count() or 1
    iters_full, how = cg_iterations_full(args.workload, n, threads)
    ref = reference_cg_seconds(case, args.warmup + args.steps, threads)
    if ref is not None:
        per_iter, it, wall = ref
        kind = "reference"
        sample = ("each step one iteration of aphros's own SolverConjugate (compiled from "
                  "its sources, blocks of 32^3, %d OpenMP threads) on the %d^3 system "
                  "assembled by aphros's Proj code; %d iterations in one run (%.3f s each, "
                  "%.0f s with the assembly); full solve = %d iterations (%s)"
                  % (threads, n, it, per_iter, wall, iters_full, how))
    else:
        e, _, _ = oracle.assemble_projection(n, h, case.dt, case.alpha, case.rho1,
                                             case.rho2, case.flux)
        for _ in range(args.warmup):
            oracle.cg_time_iters(n, e, 1, threads)
        per = [oracle.cg_time_iters(n, e, 1, threads) for _ in range(args.steps)]
        per_iter = float(np.median(per))
        kind = "port"
        sample = ("each step one CG iteration at %d^3 (C restatement of aphros "
                  "SolverConjugate, %d threads); full solve = %d iterations (%s)"
                  % (n, threads, iters_full, how))
    value = 1.0 / (per_iter * iters_full)
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_iter * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded bubble field, Taylor-Green + noise)",
        "config": {"workload": WORKLOADS[args.workload], "cells": case.N},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "cpu": cpu_model(), "cg_iters_full": iters_full, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_serve(args):
    """Served stream (C5): Poisson-arrival step requests for resident
    simulations of edge 32-128 (log-uniform, multiples of 16, 1-8 bubbles,
    density ratio 1000) on a continuous-batching server under an HBM budget,
    saturated and at each mean rate of `rates`; against the same requests
    run one at a time with the plain FP64 solver."""
    import random

    from aphros_gb300 import _lib, build, serve, workload
    build.build()
    t_setup = time.perf_counter()
    cases = workload.served_cases(args.sims)
    dts = [0.5 * c.cfl_dt(0.5) for c in cases]
    rng = random.Random(5)

    def requests(k):
        return [rng.randrange(len(cases)) for _ in range(k)]

    def drive(srv, sims, order, rate):
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
        lat = np.array([r.latency_ms for r in res])
        ok = all(r.status == _lib.OK and r.converged for r in res)
        return {"requests": len(res), "steps_per_s": len(res) / (t1 - t0),
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "all_converged": ok}

    def server(slots, conf):
        srv = serve.Server(budget_bytes=args.budget_gb * 1e9, slots=slots, conf=conf)
        sims = [srv.add(c, sigma=0.05) for c in cases]
        return srv, sims

    mixed = _lib.default_conf(solver=_lib.SOLVER_MIXED, rtol=1e-10)
    plain = _lib.default_conf(solver=_lib.SOLVER_MGPCG, rtol=1e-10)
    srv, sims = server(args.slots, mixed)
    # warm-up: one step of every simulation (admission, hierarchy, evictions)
    for t in [srv.submit(sims[i], cases[i].flux, dts[i]) for i in range(len(cases))]:
        srv.wait(t)
    setup_s = time.perf_counter() - t_setup
    saturated = drive(srv, sims, requests(args.requests), 0.0)
    rates = {}
    for rate in args.rates:
        rates[str(int(rate) if rate == int(rate) else rate)] = drive(
            srv, sims, requests(args.requests), rate)
    st = srv.stats()
    srv.close()
    # the plain FP64 solver, one request at a time, on a sample of requests
    srv1, sims1 = server(1, plain)
    order1 = requests(max(16, args.requests // 4))
    for i in sorted(set(order1)):
        srv1.wait(srv1.submit(sims1[i], cases[i].flux, dts[i]))
    one_by_one = drive(srv1, sims1, order1, 0.0)
    srv1.close()
    cells = [c.N for c in cases]
    return {
        "metric": "served steps/s and p50/p99 step latency (projection + PLIC advection + "
                  "curvature per step)",
        "value": saturated["steps_per_s"], "unit": "steps/s", "n_gpus": 1,
        "higher_is_better": True,
        "config": {"workload": "served stream, %d resident simulations of edge 32-128 "
                               "(log-uniform, multiples of 16), 1-8 bubbles, density ratio "
                               "1000, %d requests per rate, %d slots, %g GB budget"
                               % (len(cases), args.requests, args.slots, args.budget_gb),
                   "cells_total": int(sum(cells)), "cells_mean": float(np.mean(cells))},
        "served_saturated": saturated, "served_at_rate": rates,
        "one_by_one_plain_fp64": one_by_one,
        "speedup_vs_one_by_one": saturated["steps_per_s"] / one_by_one["steps_per_s"],
        "evictions": int(st.evictions), "admissions": int(st.admissions),
        "resident_gb": st.resident_bytes / 1e9, "setup_s": setup_s,
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
    if args.sweeps is not None:
        ctx.set_option(_lib.OPT_FUSED_SWEEPS, args.sweeps)
    if args.cycle == 1:
        # the benchmark line's V-cycle variant (1+1 on the finest level, 2^l
        # below; inner PCG to 1e-3 for the mixed solver)
        set_v_cycle(ctx, _lib)
        mg = dict(V_CYCLE_MG) if solver == _lib.SOLVER_MIXED else {"mg_pre": 1, "mg_post": 1}
        conf = _lib.default_conf(solver=solver, tol=tol, **mg)
    else:
        ctx.set_option(_lib.OPT_CYCLE, args.cycle)
        conf = _lib.default_conf(solver=solver, tol=tol)
    if args.profile == "vof":
        # one solve, the corrected fluxes, then `warmup` + `steps` PLIC steps
        # with the height curvature and the recolouring after each (as the
        # VOF measurement of the benchmark line)
        ctx.solve_resident(conf, zero_guess=True)
        ctx.flux_correct(out=False)
        ctx.vof_init(case.alpha)
        dt = case.cfl_dt(0.5)
        for _ in range(args.warmup + args.steps):
            ctx.vof_step(None, dt)
            ctx.curvature(out=False)
            ctx.vof_recolor()
        if args.estimator != "heights":
            # one call of the particle-string (or hybrid) estimator at the end
            est = _lib.CURV_PARTICLES if args.estimator == "particles" else _lib.CURV_HYBRID
            ctx.curvature_estimator(est, out=False)
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
    ap.add_argument("--no-v-cycle", action="store_true",
                    help="skip the V-cycle measurement beside the headline")
    ap.add_argument("--no-vof", action="store_true",
                    help="skip the PLIC advection + curvature measurement")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--cycle", type=int, choices=[0, 1, 2], default=0,
                    help="--profile: 0 library defaults (the headline; batch: the "
                         "per-domain coarse cycle), 1 the V-cycle variant, 2 W on every "
                         "level")
    ap.add_argument("--profile", choices=["mixed", "fp64", "batch", "vof"], default=None,
                    help="profiling run: assemble, then `steps` solves of one solver "
                         "after `warmup` solves, no other work and no output line")
    ap.add_argument("--sweeps", type=int, choices=[0, 1, 2, 3, 4, 5, 6], default=None,
                    help="--profile: red-black sweep variant (APHGPU_OPT_FUSED_SWEEPS)")
    ap.add_argument("--estimator", choices=["heights", "particles", "hybrid"],
                    default="heights",
                    help="--profile vof: one call of this curvature estimator after the steps")
    ap.add_argument("--serve", action="store_true",
                    help="served-stream benchmark instead of the solve benchmark")
    ap.add_argument("--sims", type=int, default=2000)
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--rates", type=float, nargs="*",
                    default=[50.0, 200.0, 500.0, 1000.0, 2000.0])
    ap.add_argument("--no-pipeline", action="store_true",
                    help="skip the C2 100-step pipeline sub-result")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the C4 batched sub-result")
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the C5 served sub-result")
    ap.add_argument("--serve-sims", type=int, default=2000)
    ap.add_argument("--serve-requests", type=int, default=256)
    ap.add_argument("--serve-rates", type=float, nargs="*",
                    default=[50.0, 200.0, 500.0, 1000.0, 2000.0])
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
