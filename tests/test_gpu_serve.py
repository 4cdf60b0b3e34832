"""Serving loop (aphgpu_server_*): each simulation's result is the same alone
and in a concurrent mix, and after eviction to host memory and restore;
admission keeps the resident device memory within the budget; a served step
agrees with the oracle (aphros's Proj assembly, CG and Vof step restated)."""
import os

import numpy as np
import pytest

import oracle
from aphros_gb300 import _lib, serve, workload

pytestmark = pytest.mark.gpu


def _cases():
    out = []
    for i, n in enumerate((24, 32, 40, 32, 24, 48)):
        c, r = workload.place_spheres(100 + i, 1 + i % 3, 0.08, 0.2, gap=0.02)
        out.append(workload.Case(n, c, r, rho1=1.0, rho2=1e-3, seed=200 + i))
    return out


def _run(cases, order, slots, budget, steps=3, sigma=0.05):
    """Submits `steps` steps of the simulations in `order` (indices into
    cases), round-robin, and returns the final states."""
    with serve.Server(budget_bytes=budget, slots=slots) as srv:
        sims = {i: srv.add(cases[i], sigma=sigma) for i in order}
        tickets = []
        for _ in range(steps):
            for i in order:
                c = cases[i]
                dt = 0.5 * c.cfl_dt(0.5)
                tickets.append(srv.submit(sims[i], c.flux, dt))
        res = []
        for t in tickets:
            try:
                res.append(srv.wait(t, timeout_s=120))
            except _lib.AphgpuError as e:
                st = srv.stats()
                raise AssertionError(
                    "ticket %d not done (%s): completed %d queued %d resident %d "
                    "resident_bytes %d budget %d evictions %d admissions %d"
                    % (t, e, st.completed, st.queued, st.resident, st.resident_bytes,
                       st.budget_bytes, st.evictions, st.admissions))
        assert all(r.status == _lib.OK for r in res)
        assert all(r.converged for r in res)
        states = {i: srv.state(sims[i]) for i in order}
        return states, res, srv.stats()


def test_alone_and_in_the_mix_are_identical():
    cases = _cases()
    alone, res_alone, _ = _run(cases, [2], slots=1, budget=100e9)
    mixed, res_mix, st = _run(cases, list(range(len(cases))), slots=4, budget=100e9)
    a0, p0 = alone[2]
    a1, p1 = mixed[2]
    assert np.array_equal(a0, a1)
    assert np.array_equal(p0, p1)
    assert st.completed == 3 * len(cases)
    assert st.evictions == 0


def test_eviction_and_restore_are_exact():
    cases = _cases()
    order = list(range(len(cases)))
    big, _, st_big = _run(cases, order, slots=2, budget=100e9)
    # room for about half of the simulations' measured device memory, and for
    # the admission estimate of the largest one (440 B/cell + 1 MiB): forces
    # evictions
    assert st_big.evictions == 0 and st_big.resident_bytes > 0
    budget = max(0.5 * st_big.resident_bytes, 1.05 * (440 * 48 ** 3 + 2 ** 20))
    assert budget < st_big.resident_bytes
    small, _, st_small = _run(cases, order, slots=2, budget=budget)
    assert st_small.evictions > 0
    assert st_small.resident_bytes <= st_small.budget_bytes
    for i in order:
        assert np.array_equal(big[i][0], small[i][0])
        assert np.array_equal(big[i][1], small[i][1])


def test_server_step_equals_manual_step():
    """A served step is the same sequence as the C-ABI calls on a context."""
    c = _cases()[1]
    dt = 0.5 * c.cfl_dt(0.5)
    states, _, _ = _run([c], [0], slots=1, budget=100e9, steps=1, sigma=0.0)
    ctx = _lib.Context(c.n, c.h)
    ctx.vof_init(c.alpha)
    ctx.assemble_projection(None, c.rho1, c.rho2, c.flux, dt)
    ctx.solve_resident(_lib.default_conf(solver=_lib.SOLVER_MIXED, rtol=1e-10))
    ctx.flux_correct(out=False)
    ctx.vof_step(None, dt)
    assert np.array_equal(ctx.vof_get()[0], states[0][0])
    assert np.array_equal(ctx.get_solution(), states[0][1])


def test_oversized_simulation_is_rejected():
    c = _cases()[5]
    with serve.Server(budget_bytes=1e6, slots=1) as srv:
        with pytest.raises(_lib.AphgpuError):
            srv.add(c)


def test_served_step_matches_oracle():
    """One served step (projection and PLIC advection, no surface tension)
    of a 32^3 simulation against the oracle on the same inputs: the pressure
    within 1e-9 (relative L2, mean removed) of the oracle's CG solved to
    ||r||/||b|| = 1e-13, and the volume fraction within 1e-12 of the
    oracle's Vof step driven by the fluxes the oracle corrects with the
    served pressure (the flux correction itself is bit-exact)."""
    c = _cases()[1]
    dt = 0.5 * c.cfl_dt(0.5)
    states, _, _ = _run([c], [0], slots=1, budget=100e9, steps=1, sigma=0.0)
    u_s, p_s = states[0][0], states[0][1]
    e, fk, fv = oracle.assemble_projection(c.n, c.h, dt, c.alpha, c.rho1, c.rho2, c.flux)
    tol = oracle.rel_tol(e, c.h, 1e-13)
    x, info = oracle.cg_solve(c.n, c.h, e, tol, nthreads=os.cpu_count() or 1)
    assert info.residual < tol
    a, b = p_s - p_s.mean(), x - x.mean()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-9
    st = oracle.VofState(c.n, c.h, c.alpha)
    st.step(oracle.flux_correct(c.n, fk, fv, p_s), dt)
    assert np.max(np.abs(st.u - u_s)) <= 1e-12
