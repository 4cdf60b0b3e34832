"""GPU parity of the pressure Poisson path against the oracle and aphros's
own outputs (golden fixtures).  Calls go through the C ABI (ctypes).

Tolerances: the projection assembly and the flux correction are bit-exact;
solutions are compared after mean removal (the periodic operator fixes p up
to a constant) in relative L2 norm: <= 1e-9 for the plain FP64 CG against
aphros's CG, both at ||r||/||b|| = 1e-10, and <= 1e-9 for MG-PCG / mixed
precision solved to ||r||/||b|| = 1e-12 against the oracle CG solved to the
same level (the error bound at 1e-10 is recorded separately).
"""
import math
import os

import numpy as np
import pytest

import oracle
from aphros_gb300 import _lib, linear, workload
from conftest import golden

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = a - a.mean()
    b = b - b.mean()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def proj16():
    return np.load(golden("proj16.npz"))


def _ctx16(fx):
    n, h = int(fx["n"]), float(fx["h"])
    ctx = _lib.Context(n, h)
    ctx.assemble_projection(fx["alpha"], float(fx["rho1"]), float(fx["rho2"]),
                            fx["vflux"], float(fx["dt"]))
    return ctx


def test_assembly_bit_exact(proj16):
    """P1-P5 fused on the device equal aphros's Proj::GetFlux/GetFluxSum
    system bit for bit (RHS mean removed)."""
    ctx = _ctx16(proj16)
    e = ctx.get_system_expr()
    ref = proj16["expr_ref"]
    # the mean of e7 is summed in a different order on the device
    mask = np.ones(8, bool)
    mask[7] = False
    assert np.array_equal(e.reshape(-1, 8)[:, mask], ref.reshape(-1, 8)[:, mask])
    assert np.max(np.abs(e[7::8] - ref[7::8])) <= 1e-17 * np.max(np.abs(ref[7::8])) + 1e-30


def test_cg_matches_reference_cg(proj16):
    """Plain FP64 CG (the algorithm of SolverConjugate) against aphros's CG
    on the same system and stopping rule."""
    ctx = _ctx16(proj16)
    conf = _lib.default_conf(solver=_lib.SOLVER_CG, tol=float(proj16["tol"]),
                             maxiter=100000)
    x, info = ctx.solve(conf)
    assert info.converged
    # CG on this system (density ratio 1000) is sensitive to the order of
    # its dot-product sums: aphros's own count changes with the block layout
    # (iters vs iters_blocks8 in the fixture).  The pressure is the gate.
    ref_iters = int(proj16["iters"])
    spread = abs(int(proj16["iters_blocks8"]) - ref_iters)
    assert abs(info.iter - ref_iters) <= max(3 * spread, ref_iters // 10)
    assert rel_l2(x, proj16["p_ref"]) <= 1e-9
    assert rel_l2(proj16["p_blocks8"], proj16["p_ref"]) <= 1e-9


@pytest.mark.parametrize("solver", [_lib.SOLVER_MGPCG, _lib.SOLVER_MIXED])
def test_multigrid_solvers_match_reference(proj16, solver):
    n, h = int(proj16["n"]), float(proj16["h"])
    ctx = _ctx16(proj16)
    e = proj16["expr_ref"]
    b = -e[7::8]
    tol12 = 1e-12 * math.sqrt(float(b @ b) / h ** 3)
    conf = _lib.default_conf(solver=solver, tol=tol12, maxiter=500)
    x, info = ctx.solve(conf)
    assert info.converged, info.residual
    xo, _ = oracle.cg_solve(n, h, e, tol12)
    assert rel_l2(x, xo) <= 1e-9
    # at the production tolerance (||r||/||b|| = 1e-10) the pressure is
    # within 1e-9 of the tight solution
    conf.tol = float(proj16["tol"])
    x10, info10 = ctx.solve(conf)
    assert info10.converged
    assert rel_l2(x10, xo) <= 1e-9


def test_expr_path_equals_assembly_path(proj16):
    """The linear::Solver drop-in (Expr AoS input) solves the same operator
    as the fused assembly: identical solutions."""
    ctx = _ctx16(proj16)
    conf = _lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=float(proj16["tol"]))
    x1, i1 = ctx.solve(conf)
    ctx2 = _lib.Context(int(proj16["n"]), float(proj16["h"]))
    ctx2.set_system_expr(ctx.get_system_expr())
    x2, i2 = ctx2.solve(conf)
    assert i1.iter == i2.iter
    assert np.array_equal(x1, x2)


def test_drop_in_solver_interface(proj16):
    """aphros_gb300.linear mirrors linear::Solver::Solve: fc_init may alias
    fc_sol, the result is written in place."""
    m = linear.Mesh(int(proj16["n"]), float(proj16["h"]))
    var = {"linsolver_symm": "gpu", "hypre_symm_tol": repr(float(proj16["tol"])),
           "hypre_symm_maxiter": "200"}
    solver = linear.MakeLinearSolver(var, "symm", m)
    sol = np.zeros(m.ncells())
    info = solver.Solve(proj16["expr_ref"], sol, sol, m)
    assert info.converged and info.residual < float(proj16["tol"])
    e = proj16["expr_ref"]
    xo, _ = oracle.cg_solve(m.n, m.h, e, oracle.rel_tol(e, m.h, 1e-13))
    assert rel_l2(sol, xo) <= 1e-9


def test_non_symmetric_system_is_rejected(proj16):
    e = proj16["expr_ref"].copy()
    e[8 * 5 + 2] *= 1.5
    ctx = _lib.Context(int(proj16["n"]), float(proj16["h"]))
    with pytest.raises(_lib.AphgpuError) as err:
        ctx.set_system_expr(e)
    assert err.value.code == _lib.ERR_NOT_SYMMETRIC


def test_flux_correction_bit_exact(proj16):
    """Proj::Project flux update on the GPU's own pressure equals the
    oracle's formula bit for bit; with aphros's pressure the fluxes agree to
    the solver tolerance."""
    n, h = int(proj16["n"]), float(proj16["h"])
    ctx = _ctx16(proj16)
    conf = _lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=float(proj16["tol"]))
    x, _ = ctx.solve(conf)
    f = ctx.flux_correct()
    _, fk, fv = oracle.assemble_projection(n, h, float(proj16["dt"]), proj16["alpha"],
                                           float(proj16["rho1"]), float(proj16["rho2"]),
                                           proj16["vflux"])
    assert np.array_equal(f, oracle.flux_correct(n, fk, fv, x))
    # corrected fluxes are discretely divergence-free to the residual level
    F = f.reshape(3, n, n, n)
    div = (np.roll(F[0], -1, axis=2) - F[0] + np.roll(F[1], -1, axis=1) - F[1]
           + np.roll(F[2], -1, axis=0) - F[2])
    assert np.max(np.abs(div)) < 1e-8 * np.max(np.abs(proj16["vflux"]))


def test_acceleration_bit_exact(proj16):
    n, h = int(proj16["n"]), float(proj16["h"])
    ctx = _ctx16(proj16)
    x, _ = ctx.solve(_lib.default_conf(tol=float(proj16["tol"])))
    acc = ctx.acceleration()
    ref = oracle.acceleration(n, h, x, proj16["alpha"], float(proj16["rho1"]),
                              float(proj16["rho2"]))
    assert np.array_equal(acc, ref)


def _diffusion_system(n, seed=3, shift=0.3):
    """A symmetric 7-point system with an explicit diagonal (the shape of
    the implicit-diffusion systems Proj also hands to linsolver_symm)."""
    N = n ** 3
    rng = np.random.default_rng(seed)
    w = -rng.uniform(0.1, 10.0, size=(3, N))
    e = np.zeros((N, 8))
    idx = np.arange(N).reshape(n, n, n)
    for d, axis in ((0, 2), (1, 1), (2, 0)):
        e[:, 1 + 2 * d] = w[d]
        e[:, 2 + 2 * d] = w[d][np.roll(idx, -1, axis=axis).ravel()]
    e[:, 0] = -e[:, 1:7].sum(axis=1) + shift
    e[:, 7] = rng.normal(size=N)
    return e.ravel()


@pytest.mark.parametrize("solver", [_lib.SOLVER_CG, _lib.SOLVER_MGPCG, _lib.SOLVER_MIXED])
def test_diffusion_type_system(solver):
    n, h = 16, 1 / 16
    e = _diffusion_system(n)
    tol = oracle.rel_tol(e, h, 1e-11)
    xo, io = oracle.cg_solve(n, h, e, tol)
    ctx = _lib.Context(n, h)
    ctx.set_system_expr(e)
    x, info = ctx.solve(_lib.default_conf(solver=solver, tol=tol, maxiter=5000))
    assert info.converged
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-9


@pytest.mark.parametrize("solver", [_lib.SOLVER_CG, _lib.SOLVER_MGPCG, _lib.SOLVER_MIXED])
@pytest.mark.parametrize("shift", [0.0, 0.5])
def test_negative_definite_system(solver, shift):
    """aphros's own Laplacian has a negative diagonal and positive couplings
    (its linear-solver test assembles it so): the system is stored negated,
    which leaves the solution and the residual norms unchanged, and reads
    back as it was set."""
    n, h = 16, 1 / 16
    e = _diffusion_system(n, shift=shift).reshape(-1, 8)
    if shift == 0:  # singular: a consistent right-hand side
        e[:, 7] -= e[:, 7].mean()
    e = e.ravel()
    tol = oracle.rel_tol(e, h, 1e-11)
    xo, _ = oracle.cg_solve(n, h, e, tol)
    ctx = _lib.Context(n, h)
    ctx.set_system_expr(-e)
    assert np.array_equal(ctx.get_system_expr(), -e)
    x, info = ctx.solve(_lib.default_conf(solver=solver, tol=tol, maxiter=5000))
    assert info.converged
    if shift == 0:  # singular: the solution up to a constant
        x = x - x.mean() + xo.mean()
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-9


@pytest.mark.parametrize("n", [24, 48])
def test_c1_sizes_and_warm_start(n):
    """Non-power-of-two grids coarsen to small odd levels; a warm start from
    the converged pressure converges immediately (miniter = 1)."""
    case = workload.config("c1", n=n)
    ctx = _lib.Context(n, case.h)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    r0, b = ctx.residual_norms()
    tol = 1e-10 * b / math.sqrt(case.h ** 3)
    for solver in (_lib.SOLVER_MGPCG, _lib.SOLVER_MIXED):
        x, info = ctx.solve(_lib.default_conf(solver=solver, tol=tol))
        assert info.converged
        rn, bn = ctx.residual_norms()
        assert rn / bn < 1.2e-10
    info = ctx.solve_resident(_lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=tol),
                              zero_guess=False)
    assert info.iter == 1


def test_full_size_property_256():
    """At 256^3 (C2: 16 bubbles, ratio 1000) both multigrid solvers reach
    ||r||/||b|| <= 1e-10 (recomputed in FP64) with the pressure within 1e-9
    of a tight FP64 solve (MG-PCG to 1e-13, W-cycle)."""
    case = workload.config("c2")
    ctx = _lib.Context(case.n, case.h)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    _, b = ctx.residual_norms()
    tol = 1e-10 * b / math.sqrt(case.h ** 3)
    ctx.set_option(_lib.OPT_CYCLE, 2)
    xt, it = ctx.solve(_lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=1e-3 * tol))
    rn, bn = ctx.residual_norms()
    assert it.converged and rn / bn <= 1.01e-13
    ctx.set_option(_lib.OPT_CYCLE, 0)
    x64, i64 = ctx.solve(_lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=tol))
    rn, bn = ctx.residual_norms()
    assert i64.converged and rn / bn <= 1.01e-10
    x32, i32 = ctx.solve(_lib.default_conf(solver=_lib.SOLVER_MIXED, tol=tol))
    rn, bn = ctx.residual_norms()
    assert i32.converged and rn / bn <= 1.01e-10
    assert rel_l2(x64, xt) <= 1e-9
    assert rel_l2(x32, xt) <= 1e-9


@pytest.mark.parametrize("solver", [_lib.SOLVER_MIXED, _lib.SOLVER_MGPCG32])
@pytest.mark.parametrize("shape", [(64, 64, 64), (96, 48, 40), (40, 24, 32), (128, 128, 128)])
def test_fused_sweeps_bit_identical(solver, shape):
    """The fused out-of-place red-black sweeps -- the pipelined kernel fed
    by asynchronous copies (mode 2: on every level with nx % 4 == 0, nx >=
    16 and nz >= 8; mode 1: on such levels of at least 2^21 cells) and the
    synchronous kernel (mode 3) -- compute every value with the operations
    of the two in-place half sweeps (mode 0), and so does the in-place
    wavefront sweep (modes 5 and 6) with any number of planes per step
    (whole chunks, a ragged last chunk, one chunk for the whole level):
    whole solves agree bit for bit (with and without CUDA graphs)."""
    nx, ny, nz = shape
    h = 1.0 / nx
    c, r = workload.place_spheres(11, 3, 0.1, 0.2, gap=0.02)
    case = workload.Case(nx, c, r, rho1=1.0, rho2=1e-3, seed=12)
    ctx = _lib.Context(shape, h)
    # the fused sweep reads the FP32 couplings: compare against the FP32
    # half sweeps in the natural order
    ctx.set_option(_lib.OPT_HALF_COUPLINGS, 0)
    ctx.set_option(_lib.OPT_COLOR_SPLIT, 0)
    N = nx * ny * nz
    alpha = workload.alpha_spheres(nx, c, r)[:N] if nx == ny == nz else np.zeros(N)
    flux = workload.tg_flux(max(shape), seed=5)
    flux = np.concatenate([flux[d * max(shape) ** 3:d * max(shape) ** 3 + N] for d in range(3)])
    ctx.assemble_projection(alpha, case.rho1, case.rho2, flux, 1e-3)
    _, bn = ctx.residual_norms()
    conf = _lib.default_conf(solver=solver, tol=1e-10 * bn / math.sqrt(h ** 3), maxiter=200)
    out = {}
    for fused in (2, 1, 4, 3, 6, 5, 0):
        for graphs in (1, 0):
            ctx.set_option(_lib.OPT_FUSED_SWEEPS, fused)
            ctx.set_option(_lib.OPT_GRAPHS, graphs)
            x, info = ctx.solve(conf)
            assert info.converged
            out[(fused, graphs)] = (x, info.iter, info.inner_iter)
    for planes in (1, 3, 5, 64):
        ctx.set_option(_lib.OPT_FUSED_SWEEPS, 6)
        ctx.set_option(_lib.OPT_GRAPHS, 1)
        ctx.set_option(_lib.OPT_WAVE_PLANES, planes)
        x, info = ctx.solve(conf)
        assert info.converged
        out[("wave", planes)] = (x, info.iter, info.inner_iter)
    ctx.set_option(_lib.OPT_WAVE_PLANES, 0)
    ref = out[(0, 0)]
    for key, val in out.items():
        assert np.array_equal(val[0], ref[0]), key
        assert val[1:] == ref[1:], key


@pytest.mark.parametrize("n", [64, 96])
def test_half_couplings_preconditioner(n):
    """The FP16 copy of the finest couplings changes only the preconditioner:
    the mixed solve reaches the same residual with the same outer iteration
    count, and the pressures agree to the solver tolerance.  The rounding of
    the couplings to 11 bits makes the finest smoother inconsistent with the
    FP32 operator by about 1e-3, which costs inner iterations (13 -> 19 at
    64^3 with a coarse series weight of 80)."""
    case = workload.config("c1", n=n)
    ctx = _lib.Context(n, case.h)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    _, bn = ctx.residual_norms()
    conf = _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=1e-10 * bn / math.sqrt(case.h ** 3))
    out = {}
    for half in (1, 0):
        ctx.set_option(_lib.OPT_HALF_COUPLINGS, half)
        x, info = ctx.solve(conf)
        rn, bn2 = ctx.residual_norms()
        assert info.converged and rn / bn2 <= 1.01e-10
        out[half] = (x, info)
    assert abs(out[1][1].iter - out[0][1].iter) <= 1
    assert out[1][1].inner_iter <= 1.6 * out[0][1].inner_iter + 2
    assert rel_l2(out[1][0], out[0][0]) < 1e-7


@pytest.mark.parametrize("solver", [_lib.SOLVER_MGPCG, _lib.SOLVER_MIXED])
def test_coarse_series_weight(solver):
    """The coarse operators' series weight (APHGPU_OPT_COARSE_SERIES) changes
    only the preconditioner: every weight reaches ||r||/||b|| <= 1e-10 on a
    64-bubble field at density ratio 1000 with the same pressure, and the
    default blend needs fewer iterations than the half-Galerkin operator
    alone (weight 0).  Out-of-range weights are rejected."""
    case = workload.config("c3", n=128)
    ctx = _lib.Context(case.n, case.h)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    _, bn = ctx.residual_norms()
    conf = _lib.default_conf(solver=solver, tol=1e-10 * bn / math.sqrt(case.h ** 3),
                             maxiter=500)
    out = {}
    for w in (0, 100, 60):
        ctx.set_option(_lib.OPT_COARSE_SERIES, w)
        x, info = ctx.solve(conf)
        rn, bn2 = ctx.residual_norms()
        assert info.converged and rn / bn2 <= 1.01e-10, w
        out[w] = (x, info.inner_iter if solver == _lib.SOLVER_MIXED else info.iter)
    for w in (0, 100):
        assert rel_l2(out[w][0], out[60][0]) < 1e-7, w
    assert out[60][1] < out[0][1]
    for bad in (-1, 101):
        with pytest.raises(_lib.AphgpuError):
            ctx.set_option(_lib.OPT_COARSE_SERIES, bad)


@pytest.mark.parametrize("cycle", [1, 2])
def test_sweep_growth(cycle):
    """More smoothing sweeps below the finest level (APHGPU_OPT_SWEEP_GROWTH)
    change only the preconditioner: every growth reaches the tolerance with
    the same pressure, and with V-cycles the linear growth needs fewer
    iterations than none."""
    case = workload.config("c3", n=128)
    ctx = _lib.Context(case.n, case.h)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    ctx.set_option(_lib.OPT_CYCLE, cycle)
    _, bn = ctx.residual_norms()
    tol = 1e-10 * bn / math.sqrt(case.h ** 3)
    out = {}
    for growth in (1, 2, 3, 0):
        ctx.set_option(_lib.OPT_SWEEP_GROWTH, growth)
        for solver in (_lib.SOLVER_MGPCG, _lib.SOLVER_MIXED):
            x, info = ctx.solve(_lib.default_conf(solver=solver, tol=tol, maxiter=300))
            rn, bn2 = ctx.residual_norms()
            assert info.converged and rn / bn2 <= 1.01e-10, (growth, solver)
            out[(growth, solver)] = (x, info.iter if solver == _lib.SOLVER_MGPCG else info.inner_iter)
    ref = out[(1, _lib.SOLVER_MGPCG)][0]
    for key, (x, _) in out.items():
        assert rel_l2(x, ref) < 1e-7, key
    if cycle == 1:
        assert out[(2, _lib.SOLVER_MGPCG)][1] < out[(1, _lib.SOLVER_MGPCG)][1]
    with pytest.raises(_lib.AphgpuError):
        ctx.set_option(_lib.OPT_SWEEP_GROWTH, 4)


@pytest.mark.parametrize("cycle", [1, 2])
@pytest.mark.parametrize("shape", [(128, 128, 128), (96, 48, 40)])
def test_cta_coarse_cycle(cycle, shape):
    """The smallest FP32 levels cycled by one CTA (APHGPU_OPT_CTA_COARSE)
    run the same smoothing, restriction, prolongation and dense coarsest
    solve as the launched passes: the mixed and MG-PCG32 solves reach the
    tolerance with the same pressure and (rounding aside) the same
    iteration counts, with and without CUDA graphs."""
    nx, ny, nz = shape
    h = 1.0 / nx
    c, r = workload.place_spheres(21, 6, 0.06, 0.15, gap=0.02)
    N = nx * ny * nz
    alpha = workload.alpha_spheres(nx, c, r)[:N] if nx == ny == nz else np.zeros(N)
    flux = workload.tg_flux(max(shape), seed=7)
    flux = np.concatenate([flux[d * max(shape) ** 3:d * max(shape) ** 3 + N] for d in range(3)])
    ctx = _lib.Context(shape, h)
    ctx.assemble_projection(alpha, 1.0, 1e-3, flux, 1e-3)
    ctx.set_option(_lib.OPT_CYCLE, cycle)
    _, bn = ctx.residual_norms()
    tol = 1e-10 * bn / math.sqrt(h ** 3)
    for solver in (_lib.SOLVER_MIXED, _lib.SOLVER_MGPCG32):
        out = {}
        for cta in (0, 1):
            for graphs in (1, 0):
                ctx.set_option(_lib.OPT_CTA_COARSE, cta)
                ctx.set_option(_lib.OPT_GRAPHS, graphs)
                x, info = ctx.solve(_lib.default_conf(solver=solver, tol=tol, maxiter=300))
                rn, bn2 = ctx.residual_norms()
                assert info.converged and rn / bn2 <= 1.01e-10, (solver, cta, graphs)
                out[(cta, graphs)] = (x, info.iter + info.inner_iter)
        ref = out[(0, 0)]
        for key, (x, its) in out.items():
            assert rel_l2(x, ref[0]) < 1e-7, (solver, key)
            # the last inner solve starts from a residual about 1e-6 of the
            # first, whose last bits the two paths round differently
            assert abs(its - ref[1]) <= max(3, 0.12 * ref[1]), (solver, key, its, ref[1])
        # graphs do not change the results
        assert np.array_equal(out[(1, 1)][0], out[(1, 0)][0])


@pytest.mark.parametrize("cycle", [1, 2])
@pytest.mark.parametrize("shape", [(128, 128, 128), (96, 48, 40), (16, 10, 6), (36, 24, 20)])
def test_color_split_finest_level(cycle, shape):
    """The mixed solver's finest FP32 level in the colour-split order
    (APHGPU_OPT_COLOR_SPLIT; shapes with nx % 8 == 0 and even ny, nz, and
    one, 36 x 24 x 20, that keeps the natural order) smooths, restricts and
    prolongs with the natural kernels' values; only the inner CG's FP32 dot
    products sum in another order.  The solves reach the tolerance with the
    same pressure and (rounding aside) the same iteration counts, with and
    without CUDA graphs; the split level's apply, restriction and half
    sweep agree with the natural ones through the whole solve."""
    nx, ny, nz = shape
    h = 1.0 / nx
    c, r = workload.place_spheres(31, 5, 0.08, 0.18, gap=0.02)
    N = nx * ny * nz
    alpha = workload.alpha_spheres(nx, c, r)[:N] if nx == ny == nz else np.zeros(N)
    flux = workload.tg_flux(max(shape), seed=9)
    flux = np.concatenate([flux[d * max(shape) ** 3:d * max(shape) ** 3 + N] for d in range(3)])
    ctx = _lib.Context(shape, h)
    ctx.set_option(_lib.OPT_HALF_COUPLINGS, 0)
    ctx.assemble_projection(alpha, 1.0, 1e-3, flux, 1e-3)
    ctx.set_option(_lib.OPT_CYCLE, cycle)
    _, bn = ctx.residual_norms()
    tol = 1e-10 * bn / math.sqrt(h ** 3)
    ctx.set_option(_lib.OPT_COLOR_SPLIT, 1)
    ctx.set_option(_lib.OPT_FUSED_SWEEPS, 0)
    ctx.set_option(_lib.OPT_GRAPHS, 0)
    ctx.solve(_lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=1e-3 * tol, maxiter=300))
    xt = ctx.get_solution()
    out = {}
    for split in (0, 1):
        for graphs in (1, 0):
            ctx.set_option(_lib.OPT_COLOR_SPLIT, split)
            ctx.set_option(_lib.OPT_GRAPHS, graphs)
            x, info = ctx.solve(_lib.default_conf(solver=_lib.SOLVER_MIXED, tol=tol, maxiter=100))
            rn, bn2 = ctx.residual_norms()
            assert info.converged and rn / bn2 <= 1.01e-10, (split, graphs)
            assert rel_l2(x, xt) <= 1e-9, (split, graphs)
            out[(split, graphs)] = (x, info.iter, info.inner_iter)
    ref = out[(0, 0)]
    for key, (x, it, inner) in out.items():
        assert rel_l2(x, ref[0]) < 1e-9, key
        assert it == ref[1] and abs(inner - ref[2]) <= 2, (key, it, inner, ref[1:])
    # graphs do not change the split path's results
    assert np.array_equal(out[(1, 1)][0], out[(1, 0)][0])
    assert out[(1, 1)][1:] == out[(1, 0)][1:]
    ctx.set_option(_lib.OPT_COLOR_SPLIT, 2)


@pytest.mark.parametrize("shape", [(128, 128, 128), (96, 48, 40), (36, 24, 20), (30, 18, 22)])
def test_double_float_residual_update(shape):
    """The mixed solver's outer residual updated as r -= s A e in
    double-float arithmetic (APHGPU_OPT_DF_RESIDUAL, flux-difference
    systems; with the colour-split finest level and without it) reaches the
    1e-10 stop with the FP64 residual b - A x recomputed afterwards within
    1% of the solver's own, the same outer iteration count as the FP64
    residual, and the pressure of the tight FP64 solution within the 1e-9
    bar.  The inner counts may differ by a few: by the last outer
    iteration the residual is about 1e-6 of the first, and both its FP64
    and its updated values carry rounding of order 1e-16 |A| |x|, near FP32
    precision relative to it, so the last inner solves start from right-hand
    sides that differ in their last bits (128^3: 3 + 14 + 13 inner
    iterations against 3 + 14 + 10)."""
    nx, ny, nz = shape
    h = 1.0 / nx
    c, r = workload.place_spheres(41, 5, 0.08, 0.18, gap=0.02)
    N = nx * ny * nz
    alpha = workload.alpha_spheres(nx, c, r)[:N] if nx == ny == nz else np.zeros(N)
    flux = workload.tg_flux(max(shape), seed=13)
    flux = np.concatenate([flux[d * max(shape) ** 3:d * max(shape) ** 3 + N] for d in range(3)])
    ctx = _lib.Context(shape, h)
    ctx.assemble_projection(alpha, 1.0, 1e-3, flux, 1e-3)
    _, bn = ctx.residual_norms()
    tol = 1e-10 * bn / math.sqrt(h ** 3)
    ctx.solve(_lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=1e-3 * tol, maxiter=300))
    xt = ctx.get_solution()
    out = {}
    for split in (1, 0):
        for dfr in (1, 0):
            ctx.set_option(_lib.OPT_COLOR_SPLIT, split)
            ctx.set_option(_lib.OPT_DF_RESIDUAL, dfr)
            x, info = ctx.solve(_lib.default_conf(solver=_lib.SOLVER_MIXED, tol=tol, maxiter=100))
            rn, bn2 = ctx.residual_norms()
            assert info.converged and rn / bn2 <= 1.01e-10, (split, dfr, rn / bn2)
            # the solver's residual (updated) against b - A x in FP64
            true_res = rn / math.sqrt(h ** 3)
            assert abs(info.residual - true_res) <= 1e-2 * true_res, (split, dfr, info.residual,
                                                                    true_res)
            assert rel_l2(x, xt) <= 1e-9, (split, dfr)
            out[(split, dfr)] = (x, info.iter, info.inner_iter)
    for split in (1, 0):
        a, b = out[(split, 1)], out[(split, 0)]
        assert rel_l2(a[0], b[0]) < 1e-9, split
        assert a[1] == b[1] and abs(a[2] - b[2]) <= max(3, 0.2 * b[2]), (split, a[1:], b[1:])
    ctx.set_option(_lib.OPT_COLOR_SPLIT, 2)
    ctx.set_option(_lib.OPT_DF_RESIDUAL, 2)


@pytest.mark.parametrize("solver", [_lib.SOLVER_MIXED, _lib.SOLVER_MGPCG])
def test_w_cycle_floor(solver):
    """W-cycles whose small levels visit the level below once
    (APHGPU_OPT_W_MIN_CELLS: none, 16^3 = the default, 32^3) reach the
    1e-10 stop with the pressure of the tight FP64 solution within the
    1e-9 bar, with CUDA graphs (the floor is part of the graph's key)."""
    n = 128
    h = 1.0 / n
    c, r = workload.place_spheres(51, 5, 0.08, 0.18, gap=0.02)
    ctx = _lib.Context(n, h)
    ctx.assemble_projection(workload.alpha_spheres(n, c, r), 1.0, 1e-3,
                            workload.tg_flux(n, seed=17), 1e-3)
    _, bn = ctx.residual_norms()
    tol = 1e-10 * bn / math.sqrt(h ** 3)
    ctx.solve(_lib.default_conf(solver=_lib.SOLVER_MGPCG, tol=1e-3 * tol, maxiter=300))
    xt = ctx.get_solution()
    ctx.set_option(_lib.OPT_CYCLE, 2)
    its = {}
    for wmin in (0, 4096, 32768, 4096):
        ctx.set_option(_lib.OPT_W_MIN_CELLS, wmin)
        x, info = ctx.solve(_lib.default_conf(solver=solver, tol=tol, maxiter=300))
        rn, bn2 = ctx.residual_norms()
        assert info.converged and rn / bn2 <= 1.01e-10, wmin
        assert rel_l2(x, xt) <= 1e-9, wmin
        key = (wmin, info.iter, info.inner_iter)
        its.setdefault(wmin, key)
        assert its[wmin] == key  # the same graph key rebuilt gives the same solve
    ctx.set_option(_lib.OPT_CYCLE, 0)


@pytest.mark.parametrize("shape", [(30, 18, 22), (18, 18, 18), (26, 12, 14)])
def test_ragged_grids_scalar_paths(shape):
    """Grids whose x size is not a multiple of 4 take the scalar kernels
    (no float4 tiles) on every level; every solver still matches the
    oracle's CG to 1e-9 at ||r||/||b|| = 1e-12."""
    nx, ny, nz = shape
    h = 1.0 / nx
    N = nx * ny * nz
    rng = np.random.default_rng(nx * 100 + ny)
    # a bubble-like coefficient field: random density ratio per cell
    alpha = (rng.uniform(size=N) > 0.7).astype(np.float64)
    flux = rng.normal(size=3 * N) * h * h
    ctx = _lib.Context(shape, h)
    ctx.assemble_projection(alpha, 1.0, 1e-2, flux, 1e-3)
    e = ctx.get_system_expr()
    _, bn = ctx.residual_norms()
    tol = 1e-12 * bn / math.sqrt(h ** 3)
    xo, _ = oracle.cg_solve(shape, h, e, tol, maxiter=100000)
    for solver in (_lib.SOLVER_CG, _lib.SOLVER_MGPCG, _lib.SOLVER_MIXED, _lib.SOLVER_MGPCG32):
        x, info = ctx.solve(_lib.default_conf(solver=solver, tol=tol, maxiter=20000))
        assert info.converged, solver
        assert rel_l2(x, xo) < 1e-9, solver


def test_cell_conditions():
    """Given-pressure cells (Proj::ApplyCellCond, proj.ipp:326-338) on the
    assembled C1 system at 32^3: the modified system equals the oracle's bit
    for bit (e[7] up to the order of the mean removal), and every solver
    reaches the oracle CG's pressure (no mean removed: the system is no
    longer singular)."""
    case = workload.config("c1", n=32)
    n, h = case.n, case.h
    ctx = _lib.Context(n, h)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    e0 = ctx.get_system_expr()
    cells = np.array([0, 5 + 32 * (7 + 32 * 11), n ** 3 - 1, 16 + 32 * (16 + 32 * 16)])
    values = np.array([0.25, -1.5, 3.0, 0.0])
    ctx.apply_cell_cond(cells, values)
    e = ctx.get_system_expr()
    ref = oracle.apply_cell_cond(e0, cells, values)
    assert np.array_equal(e, ref)
    # the unit penalty beside couplings of 1e-4 .. 1e-1 makes the system
    # badly conditioned: the plain CG needs tens of thousands of iterations
    # and two solutions at ||r||/||b|| = 1e-12 differ by ~3e-9, so the
    # solutions are checked by their true residual (recomputed by the
    # oracle in FP64) and against the oracle's CG within 1e-7
    tol = oracle.rel_tol(ref, h, 1e-12)
    xo, io = oracle.cg_solve(n, h, ref, tol, nthreads=os.cpu_count() or 1)
    assert io.residual < tol
    for solver in (_lib.SOLVER_MGPCG, _lib.SOLVER_MIXED, _lib.SOLVER_CG):
        x, info = ctx.solve(_lib.default_conf(solver=solver, tol=tol, maxiter=200000))
        assert info.converged, solver
        # true residual within 10x the tolerance (the recursive residual of
        # the solvers drifts from the true one on this system)
        assert math.sqrt(oracle.residual(n, ref, x)[1]) <= 10 * tol * math.sqrt(h ** 3), solver
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= 1e-7, solver
    # a cell given twice, a cell outside the domain
    with pytest.raises(_lib.AphgpuError):
        ctx.apply_cell_cond([3, 3], [1.0, 1.0])
    with pytest.raises(_lib.AphgpuError):
        ctx.apply_cell_cond([n ** 3], [1.0])


def test_wavefront_wait_gives_up_and_reports():
    """The wavefront sweep's bounded wait, run on a progress counter that
    nothing sets, gives up and reports APHGPU_ERR_TIMEOUT (no fault, no
    hang); the context stays usable, and a following wavefront solve (whose
    waits all end) returns the half sweeps' result."""
    import time
    n = 32
    c, r = workload.place_spheres(3, 2, 0.1, 0.2, gap=0.02)
    case = workload.Case(n, c, r, rho1=1.0, rho2=1e-3, seed=4)
    ctx = _lib.Context(n, case.h)
    ctx.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    _, bn = ctx.residual_norms()
    conf = _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=1e-10 * bn / math.sqrt(case.h ** 3))
    # the half sweeps in the natural order, which the wavefront reproduces
    ctx.set_option(_lib.OPT_COLOR_SPLIT, 0)
    x0, _ = ctx.solve(conf)
    t0 = time.perf_counter()
    rc = ctx._L.aphgpu_wave_wait_check(ctx.handle)
    waited = time.perf_counter() - t0
    print("bounded wait gave up after %.2f s" % waited)
    assert rc == _lib.ERR_TIMEOUT
    assert waited < 30
    ctx.set_option(_lib.OPT_FUSED_SWEEPS, 6)
    x6, info = ctx.solve(conf)
    assert info.converged
    assert np.array_equal(x6, x0)
    ctx.close()
