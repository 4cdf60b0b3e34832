"""Connected-component colours of the volume fraction (aphgpu_vof_recolor)
against aphros's own Vof::GetColor (golden fixtures, tests/golden/colors.npz)
and against the oracle's restatement on the GPU's own volume fractions."""
import numpy as np
import pytest

import oracle
from aphros_gb300 import _lib, workload
from conftest import golden

pytestmark = pytest.mark.gpu


def test_colors_equal_reference():
    """After 1, 3 and 8 steps (a recolouring after each): separate bubbles,
    touching bubbles that merge, spheres across the periodic boundary."""
    fx = np.load(golden("colors.npz"))
    steps = [int(s) for s in fx["steps"]]
    for q in range(3):
        n = int(fx["n%d" % q])
        case = workload.Case(n, fx["centres%d" % q], fx["radii%d" % q], seed=int(fx["seed%d" % q]))
        dt = case.cfl_dt(0.5)
        ctx = _lib.Context(n, case.h)
        ctx.vof_init(case.alpha)
        assert np.array_equal(ctx.vof_colors(), np.where(case.alpha > 0, 0.0, -1.0))
        st = oracle.VofState(n, case.h, case.alpha)
        for s in range(1, max(steps) + 1):
            prev = ctx.vof_colors()
            ctx.vof_step(case.flux, dt)
            ctx.vof_recolor()
            cl = ctx.vof_colors()
            u = ctx.vof_get()[0]
            # the oracle's recolouring of the GPU's own field
            assert np.array_equal(cl, oracle.recolor(n, u, prev)), (q, s)
            st.step(case.flux, dt)
            st.recolor()
            if s in steps:
                # the oracle's field is aphros's (pinned on the CPU); the
                # GPU's agrees to round-off (not always to the last bit),
                # far from the colour thresholds here
                assert np.max(np.abs(u - st.u)) <= 1e-12, (q, s)
                assert np.array_equal(cl, fx["cl%d_%d" % (q, s)].astype(np.float64)), (q, s)
        ctx.close()


@pytest.mark.parametrize("n,count", [(128, 64), (96, 200)])
def test_colors_many_bubbles(n, count):
    """Many bubbles at 96^3-128^3: the GPU recolouring equals the oracle's
    on the same field over several steps, and every gas cell is coloured."""
    c, r = workload.place_spheres(n + count, count, 0.02, 0.06, gap=0.0)
    case = workload.Case(n, c, r, seed=3)
    dt = case.cfl_dt(0.5)
    ctx = _lib.Context(n, case.h)
    ctx.vof_init(case.alpha)
    for s in range(3):
        prev = ctx.vof_colors()
        ctx.vof_step(case.flux, dt)
        ctx.vof_recolor()
        cl = ctx.vof_colors()
        u = ctx.vof_get()[0]
        assert np.array_equal(cl, oracle.recolor(n, u, prev)), s
        assert np.all(cl[u > 0.5] >= 0)
    assert len(np.unique(cl[cl >= 0])) >= 0.3 * len(r)
    ctx.close()
