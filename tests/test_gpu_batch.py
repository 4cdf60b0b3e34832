"""Batched solve (aphgpu_batch_*): many uneven domains in shared launches.

Each domain's batched result is compared with its own mixed-precision solve
(same algorithm, different launch grouping), every domain's FP64 residual is
recomputed after the batch, a domain's result does not depend on which other
domains share the batch, and repeated solves are bit-identical."""
import math

import numpy as np
import pytest

from aphros_gb300 import _lib, workload

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _domains():
    out = []
    for i, n in enumerate((16, 24, 32, 20, 48, 32, 16, 24)):
        c, r = workload.place_spheres(300 + i, 1 + i % 4, 0.06, 0.2, gap=0.02)
        ratio = 10.0 ** (1 + 2 * ((i * 0.37) % 1.0))
        out.append(workload.Case(n, c, r, rho1=1.0, rho2=1.0 / ratio, seed=400 + i))
    return out


def _diffusion_expr(n, seed=3, shift=0.3):
    """A symmetric 7-point system with an explicit diagonal shift (the
    shape of the implicit-diffusion systems also handed to linsolver_symm)."""
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


def _contexts(cases, diffusion=True):
    ctxs = []
    for c in cases:
        ctx = _lib.Context(c.n, c.h)
        ctx.assemble_projection(c.alpha, c.rho1, c.rho2, c.flux, c.dt)
        ctxs.append(ctx)
    if diffusion:
        ctx = _lib.Context(16, 1 / 16)
        ctx.set_system_expr(_diffusion_expr(16))
        ctxs.append(ctx)
    return ctxs


def _conf(**kw):
    # tol: absolute floor (a zero right-hand side converges at once)
    return _lib.default_conf(solver=_lib.SOLVER_MIXED, tol=1e-30, rtol=RTOL, maxiter=100,
                             **kw)


def _demean(x):
    return x - x.mean()


def test_batch_equals_individual_mixed_solves():
    ctxs = _contexts(_domains())
    conf = _conf()
    ref, ref_info = [], []
    for ctx in ctxs:
        info = ctx.solve_resident(conf, zero_guess=True)
        assert info.converged
        ref.append(ctx.get_solution())
        ref_info.append(info)
    batch = _lib.Batch(ctxs)
    infos = batch.solve(conf)
    for q, (ctx, info) in enumerate(zip(ctxs, infos)):
        assert info.converged, q
        rn, bn = ctx.residual_norms()
        assert rn / bn <= 1.01 * RTOL, q
        x = ctx.get_solution()
        a, b = _demean(x), _demean(ref[q])
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-7, q
        assert abs(info.iter - ref_info[q].iter) <= 1, q
    ms, launches = batch.last()
    assert ms > 0 and launches > 0
    batch.close()


def test_alone_and_in_the_batch_are_identical():
    cases = _domains()
    conf = _conf()
    mix = _contexts(cases)
    b = _lib.Batch(mix)
    infos = b.solve(conf)
    x_mix = [c.get_solution() for c in mix]
    for q in (0, 4, len(mix) - 1):
        alone = _contexts([cases[q]], diffusion=False) if q < len(cases) else \
            _contexts([], diffusion=True)
        ba = _lib.Batch(alone)
        ia = ba.solve(conf)
        assert np.array_equal(alone[0].get_solution(), x_mix[q]), q
        assert ia[0].iter == infos[q].iter and ia[0].inner_iter == infos[q].inner_iter
        ba.close()
    b.close()


def test_repeat_is_bit_identical_and_domains_stop_independently():
    cases = _domains()[:4]
    ctxs = _contexts(cases, diffusion=False)
    # a domain with a zero right-hand side is converged before any iteration
    zero = _lib.Context(16, 1 / 16)
    assert cases[0].n == 16
    e = ctxs[0].get_system_expr().reshape(-1, 8).copy()
    e[:, 7] = 0.0
    zero.set_system_expr(e.ravel())
    ctxs.append(zero)
    batch = _lib.Batch(ctxs)
    conf = _conf(miniter=0)
    i1 = batch.solve(conf)
    x1 = [c.get_solution() for c in ctxs]
    i2 = batch.solve(conf)
    x2 = [c.get_solution() for c in ctxs]
    for a, b in zip(x1, x2):
        assert np.array_equal(a, b)
    assert [v.iter for v in i1] == [v.iter for v in i2]
    assert i1[-1].converged and i1[-1].iter == 0
    assert np.all(x1[-1] == 0.0)
    assert all(v.iter > 0 for v in i1[:-1])
    batch.close()


@pytest.mark.parametrize("planes,coarse_cells,cycle", [(1, 0, 1), (2, 512, 2), (8, 32768, 1),
                                                     (8, 32768, 2), (4, 10 ** 6, 2)])
def test_tilings_agree(planes, coarse_cells, cycle):
    """Every tiling (planes per tile; coarse levels cycled per domain from
    only the coarsest up to whole domains; V- or W-cycles there) converges
    to the same pressure."""
    ctxs = _contexts(_domains())
    conf = _conf()
    ref = []
    for ctx in ctxs:
        ctx.solve_resident(conf, zero_guess=True)
        ref.append(ctx.get_solution())
    batch = _lib.Batch(ctxs)
    batch.set_tiles(planes, coarse_cells)
    batch.set_cycle(cycle)
    assert batch.tiles() == (planes, coarse_cells) and batch.cycle() == cycle
    infos = batch.solve(conf)
    for q, (ctx, info) in enumerate(zip(ctxs, infos)):
        assert info.converged, q
        rn, bn = ctx.residual_norms()
        assert rn / bn <= 1.01 * RTOL, q
        a, b = _demean(ctx.get_solution()), _demean(ref[q])
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-7, q
    batch.close()


def test_tune_keeps_results_converged():
    ctxs = _contexts(_domains()[:5], diffusion=False)
    batch = _lib.Batch(ctxs)
    conf = _conf()
    best = batch.tune(conf)
    assert best > 0 and conf.mg_pre == conf.mg_post and 1 <= conf.mg_pre <= 3
    infos = batch.solve(conf)
    for ctx, info in zip(ctxs, infos):
        assert info.converged
        rn, bn = ctx.residual_norms()
        assert rn / bn <= 1.01 * RTOL
    batch.close()


def test_coarsest_too_large_is_rejected():
    # 2 * 17^3 cells cannot be halved (odd) and exceed the dense coarsest size
    ctx = _lib.Context((34, 34, 17), 1 / 34)
    e = np.zeros((34 * 34 * 17, 8))
    e[:, 1:7] = -1.0
    e[:, 0] = 6.0
    e[:, 7] = np.sin(np.arange(e.shape[0]))
    e[:, 7] -= e[:, 7].mean()
    ctx.set_system_expr(e.ravel())
    batch = _lib.Batch([ctx])
    with pytest.raises(_lib.AphgpuError):
        batch.solve(_conf())
    batch.close()
    assert math.isfinite(ctx.residual_norms()[1])


def test_ragged_domains_in_one_batch():
    """Domains whose x size is not a multiple of 4 (scalar tiles; they
    coarsen once, to an odd size whose cube the dense coarsest inverse
    takes) batched with float4 ones: each converges and equals its own
    mixed solve."""
    cases = []
    for i, n in enumerate((18, 14, 32, 10, 24)):
        c, r = workload.place_spheres(500 + i, 2, 0.08, 0.2, gap=0.02)
        cases.append(workload.Case(n, c, r, rho1=1.0, rho2=1e-3, seed=600 + i))
    ctxs = _contexts(cases, diffusion=False)
    conf = _conf()
    ref = []
    for ctx in ctxs:
        info = ctx.solve_resident(conf, zero_guess=True)
        assert info.converged
        ref.append(ctx.get_solution())
    batch = _lib.Batch(ctxs)
    infos = batch.solve(conf)
    for q, (ctx, info) in enumerate(zip(ctxs, infos)):
        assert info.converged, q
        rn, bn = ctx.residual_norms()
        assert rn / bn <= 1.01 * RTOL, q
        a, b = _demean(ctx.get_solution()), _demean(ref[q])
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-7, q
    batch.close()


def _c4_selection():
    """Eight domains of the 512-domain C4 draw: for every edge in
    {32, 48, 64, 96} the one with the lowest and the one with the highest
    density ratio (ratios drawn log-uniformly in [10, 1000])."""
    cases = workload.batch_cases(512)
    out = []
    for n in (32, 48, 64, 96):
        same = [c for c in cases if c.n == n]
        ratio = lambda c: c.rho1 / c.rho2
        out.append(min(same, key=ratio))
        out.append(max(same, key=ratio))
    return out


def test_batch_c4_domains_within_1e9_of_oracle_cg():
    """Each of eight C4 domains solved in one batch to ||r||/||b|| = 1e-10
    has its pressure within 1e-9 (relative L2, mean removed) of the oracle's
    CG (the algorithm of aphros's SolverConjugate) solved to 1e-13."""
    import os

    import oracle
    cases = _c4_selection()
    ratios = [c.rho1 / c.rho2 for c in cases]
    assert min(ratios) < 15 and max(ratios) > 700
    ctxs = _contexts(cases, diffusion=False)
    batch = _lib.Batch(ctxs)
    infos = batch.solve(_conf())
    for q, (c, ctx, info) in enumerate(zip(cases, ctxs, infos)):
        assert info.converged, q
        e = ctx.get_system_expr()
        tol = oracle.rel_tol(e, c.h, 1e-13)
        xo, io = oracle.cg_solve(c.n, c.h, e, tol, nthreads=os.cpu_count() or 1)
        assert io.residual < tol, q
        a, b = _demean(ctx.get_solution()), _demean(xo)
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err <= 1e-9, (q, c.n, ratios[q], err)
    batch.close()
