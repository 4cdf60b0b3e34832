"""Pins the CPU oracle against aphros itself (CPU, no GPU needed).

Every check compares the C restatement (oracle/aphros_oracle.c) with values
produced by aphros's own code: the golden fixtures made by
tests/golden/make_golden.py from oracle/_ref/ref_harness, and the
reference's committed golden files where the reference tree is present.
"""
import math
import os

import numpy as np
import pytest

import oracle
from aphros_gb300 import workload
from conftest import REFERENCE, golden, read_table


def _bits_equal(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    return np.all((a == b) | both_nan)


def test_reconst_geometry_matches_reference():
    """GetLineA / GetLineU / GetLineFlux (src/solver/reconst.h) on random
    planes: identical bits."""
    rows = read_table("reconst.txt")
    assert len(rows) >= 200
    mism = 0
    for inp, out in rows:
        v = [float(x) for x in inp.split()]
        n, u, a, h, q, dt, d = v[0:3], v[3], v[4], v[5:8], v[8], v[9], int(v[10])
        ra, ru, rf = [float(x) for x in out.split()]
        ga = oracle.line_a(n, u, h)
        gu = oracle.line_u(n, a, h)
        gf = oracle.line_flux(n, a, h, q, dt, d)
        for x, y in ((ga, ra), (gu, ru), (gf, rf)):
            if not (x == y or (math.isnan(x) and math.isnan(y))):
                mism += 1
                assert abs(x - y) <= 1e-14 * max(1.0, abs(y)), (inp, x, y)
    # libm may differ in the last bit on another platform; here it is exact
    assert mism <= len(rows) // 20


def test_reconst_identities():
    """Known answers of test/reconst/main.cpp:116-124 and u(a(u)) = u."""
    one = (1.0, 1.0, 1.0)
    assert abs(oracle.line_u((0.0, 1.0, 0.0), 0.0, one) - 0.5) < 1e-12
    assert abs(oracle.line_u((1.0, 1.0, 1.0), -1.5, one) - 0.0) < 1e-12
    assert abs(oracle.line_u((1.0, 1.0, 1.0), 1.5, one) - 1.0) < 1e-12
    assert abs(oracle.line_u((1.0, 1.0, 1.0), -0.5, one) - 1.0 / 6.0) < 1e-12
    rng = np.random.default_rng(0)
    for _ in range(2000):
        n = rng.uniform(size=3) * rng.integers(0, 2, size=3)
        if not n.any():
            n[0] = 1
        n /= np.linalg.norm(n)
        u = rng.uniform()
        h = (0.1, 0.2, 0.3)
        a = oracle.line_a(n, u, h)
        assert abs(oracle.line_u(n, a, h) - u) < 1e-10


def test_height_good_matches_reference():
    rows = read_table("height.txt")
    ntest = 0
    for inp, out, exp in rows:
        toks = inp.split()
        nn = None
        if toks[0].startswith("n="):
            nn = float(toks[0][2:])
            toks = toks[1:]
        uu = [float(t) for t in toks]
        g = oracle.height_good_n(uu, nn) if nn is not None else oracle.height_good(uu)
        r = float(out)
        assert (g == r) or (math.isnan(g) and math.isnan(r)), (inp, g, r)
        # the reference unit test's own expectation (test/util/main.cpp)
        if exp in ("true", "false"):
            assert (not math.isnan(g)) == (exp == "true")
            ntest += 1
        elif exp != "random":
            e = float(exp)
            assert (math.isnan(g) and math.isnan(e)) or abs(g - e) < 1e-6
            ntest += 1
    assert ntest >= 20


def test_generator_overlap_matches_reference():
    """Our sphere/cell overlap (workload generator) against aphros's
    GetSphereOverlap (src/overlap/overlap.cpp)."""
    g = workload.gen()
    rows = read_table("overlap.txt")
    worst = 0.0
    for inp, out in rows:
        x, y, z, hx, hy, hz, cx, cy, cz, r = [float(t) for t in inp.split()]
        ref = float(out)
        vol = g.aphgen_box_sphere(x - hx / 2 - cx, x + hx / 2 - cx, y - hy / 2 - cy,
                                  y + hy / 2 - cy, z - hz / 2 - cz, z + hz / 2 - cz, r)
        frac = vol / (hx * hy * hz)
        worst = max(worst, abs(frac - ref))
    assert worst < 1e-10, worst


def _advection3d_oracle(fx):
    n3 = tuple(int(v) for v in fx["n"])
    h = float(fx["h"])
    flux = workload.uniform_flux(n3, h, fx["vel"])
    st = oracle.VofState(n3, h, fx["u_init"])
    for _ in range(int(fx["steps"])):
        st.step(flux, float(fx["dt"]))
    return st


def test_advection3d_reference_golden():
    """The reference's own 3-D advection test (test/advection, 3d.conf):
    58 Weymouth steps of a sphere in uniform flow.  Against the committed
    golden u_0002.dat with the test's threshold 1e-11 (test/advection/test:78)
    and bit for bit against aphros run on one block."""
    fx = np.load(golden("advection3d.npz"))
    st = _advection3d_oracle(fx)
    assert np.nanmax(np.abs(st.u - fx["u_golden"])) <= 1e-11
    assert _bits_equal(st.u, fx["u_ref"])
    assert _bits_equal(st.nrm, fx["n_ref"])
    assert _bits_equal(st.a, fx["a_ref"])
    assert _bits_equal(st.curvature(), fx["k_ref"])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "src")),
                    reason="reference tree not present")
def test_advection3d_fixture_is_reference_file():
    """The fixture's golden field is the reference's file itself."""
    path = os.path.join(REFERENCE, "src/test/advection/ref/3d/u_0002.dat")
    with open(path) as f:
        f.readline()
        u2 = np.array(f.read().split(), dtype=float)
    fx = np.load(golden("advection3d.npz"))
    assert np.array_equal(u2, fx["u_golden"])


def test_projection_assembly_and_cg_match_reference():
    """Proj::GetFlux/GetFluxSum assembly and SolverConjugate on 16^3,
    density ratio 1000: identical system, identical CG iterates (the
    reference ran on one block, so its reductions are sequential too)."""
    fx = np.load(golden("proj16.npz"))
    n, h = int(fx["n"]), float(fx["h"])
    e, fk, fv = oracle.assemble_projection(n, h, float(fx["dt"]), fx["alpha"],
                                           float(fx["rho1"]), float(fx["rho2"]),
                                           fx["vflux"])
    assert _bits_equal(e, fx["expr_ref"])
    x, info = oracle.cg_solve(n, h, e, float(fx["tol"]))
    assert info.iter == int(fx["iters"])
    assert _bits_equal(x, fx["p_ref"])
    f = oracle.flux_correct(n, fk, fv, x)
    assert _bits_equal(f, fx["flux_ref"])


def test_vof32_matches_reference():
    """3 Weymouth steps (all three split orders) and Heights curvature on
    the 32^3 sphere in Taylor-Green flow."""
    fx = np.load(golden("vof32.npz"))
    case = workload.config("c1", n=int(fx["n"]))
    assert abs(case.alpha.sum() - float(fx["alpha_sum"])) < 1e-9
    st = oracle.VofState(case.n, case.h, case.alpha)
    for _ in range(int(fx["steps"])):
        st.step(case.flux, float(fx["dt"]))
    assert np.max(np.abs(st.u - fx["u_ref"])) <= 1e-13
    k = st.curvature()
    m = ~np.isnan(fx["k_ref"])
    assert np.array_equal(np.isnan(k), ~m)
    assert np.max(np.abs(k[m] - fx["k_ref"][m])) <= 1e-9


def test_sphere_curvature_close_to_exact():
    """Heights curvature of a sphere r=0.2 on 64^3 is close to 2/r = 10."""
    case = workload.config("c1", n=64)
    st = oracle.VofState(64, case.h, case.alpha)
    # reconstruct without advecting: a zero-flux step
    st.step(np.zeros(3 * case.N), 1e-3)
    k = st.curvature()
    kk = k[~np.isnan(k)]
    assert len(kk) > 1000
    assert abs(np.median(kk) - 10.0) < 0.3


def test_cg_converges_on_random_spd():
    """The oracle CG solves a small diffusion system (explicit diagonal)."""
    n = 8
    N = n ** 3
    rng = np.random.default_rng(3)
    w = -rng.uniform(0.5, 2.0, size=(3, N))
    e = np.zeros((N, 8))
    idx = np.arange(N).reshape(n, n, n)  # [k, j, i]
    for d, axis in ((0, 2), (1, 1), (2, 0)):
        e[:, 1 + 2 * d] = w[d]
        e[:, 2 + 2 * d] = w[d][np.roll(idx, -1, axis=axis).ravel()]
    e[:, 0] = -e[:, 1:7].sum(axis=1) + 0.5
    xs = rng.normal(size=N)
    r, _ = oracle.residual(n, e.ravel(), xs)  # r = -(A xs + e7) with e7 = 0
    e[:, 7] = r  # now A xs + e7 = 0
    x, info = oracle.cg_solve(n, 1.0, e.ravel(), 1e-12)
    assert np.max(np.abs(x - xs)) < 1e-8


def test_oracle_colors_equal_reference():
    """The oracle's union-find recolouring (resetcolor, recolor with the
    stable colour map, propagate) gives aphros's own Vof::GetColor after 1,
    3 and 8 steps: separate bubbles, touching bubbles that merge, and
    spheres across the periodic boundary."""
    fx = np.load(golden("colors.npz"))
    steps = [int(s) for s in fx["steps"]]
    for q in range(3):
        n = int(fx["n%d" % q])
        case = workload.Case(n, fx["centres%d" % q], fx["radii%d" % q], seed=int(fx["seed%d" % q]))
        dt = case.cfl_dt(0.5)
        st = oracle.VofState(n, case.h, case.alpha)
        for s in range(1, max(steps) + 1):
            st.step(case.flux, dt)
            cl = st.recolor()
            if s in steps:
                assert np.array_equal(cl, fx["cl%d_%d" % (q, s)].astype(np.float64)), (q, s)


def test_oracle_colors_properties():
    """Properties of the recolouring on random fields: every gas cell is
    coloured, 26-adjacent gas cells (periodic) share a colour, distinct
    components get distinct colours, and recolouring an unchanged field
    keeps every colour."""
    rng = np.random.default_rng(23)
    for n in ((12, 10, 8), (9, 9, 9)):
        u = rng.uniform(size=n[0] * n[1] * n[2])
        u[u < 0.4] = 0.0
        prev = np.where(u > 0, 0.0, -1.0)
        cl = oracle.recolor(n, u, prev)
        gas = u > 0.5
        assert np.all(cl[gas] >= 0)
        g = gas.reshape(n[2], n[1], n[0])
        c3 = cl.reshape(n[2], n[1], n[0])
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    gn = np.roll(g, (-dz, -dy, -dx), axis=(0, 1, 2))
                    cn = np.roll(c3, (-dz, -dy, -dx), axis=(0, 1, 2))
                    both = g & gn
                    assert np.array_equal(c3[both], cn[both])
        # distinct components: the colours of gas cells number the
        # components (scipy's labelling with periodic merging as the check)
        from scipy import ndimage
        lab, nlab = ndimage.label(g, structure=np.ones((3, 3, 3)))
        # merge labels across the periodic boundaries
        parent = list(range(nlab + 1))

        def find(a):
            while parent[a] != a:
                parent[a] = parent[parent[a]]
                a = parent[a]
            return a
        for ax in range(3):
            a = np.take(lab, 0, axis=ax)
            for sh in (-1, 0, 1):
                for sh2 in (-1, 0, 1):
                    b = np.take(lab, -1, axis=ax)
                    b = np.roll(np.roll(b, sh, axis=0), sh2, axis=1)
                    m = (a > 0) & (b > 0)
                    for x, y in zip(a[m], b[m]):
                        parent[find(x)] = find(y)
        ncomp = len({find(v) for v in np.unique(lab[lab > 0])})
        assert len(np.unique(cl[gas])) == ncomp
        assert np.array_equal(oracle.recolor(n, u, cl), cl)


def test_oracle_bcg_predictor_equals_reference():
    """UEmbed::InterpolateBcg (the BCG face predictor of Proj::StartStep) on
    periodic 12x10x8 and 8^3 meshes: the oracle's face values are aphros's
    bit for bit."""
    fx = np.load(golden("bcg.npz"))
    for q in range(2):
        n3 = tuple(int(v) for v in fx["n%d" % q])
        ffu = oracle.interpolate_bcg(n3, float(fx["h%d" % q]), fx["u%d" % q], fx["vflux%d" % q],
                                     fx["src%d" % q], float(fx["dt%d" % q]))
        assert np.array_equal(ffu, fx["ffu%d" % q]), q


def test_oracle_fluid_step_equals_reference():
    """The oracle's projection fluid step (Proj with the default ProjPar:
    initial pressure, BCG predictor and its projection, advection, implicit
    diffusion, projection, acceleration) gives aphros's velocity, pressure
    and face fluxes bit for bit after 1 and 4 steps (digests of aphros's
    own run, tests/golden/fluid.npz)."""
    import hashlib
    import sys
    sys.path.insert(0, os.path.dirname(golden("fluid.npz")))
    from make_golden import FLUID, taylor_green_cells
    fx = np.load(golden("fluid.npz"))
    steps = [int(s) for s in fx["steps"]]
    for q in range(2):
        n = int(fx["n%d" % q])
        case = workload.Case(n, fx["centres%d" % q], fx["radii%d" % q], seed=1)
        a = case.alpha
        rho = FLUID["rho1"] * (1 - a) + FLUID["rho2"] * a
        mu = FLUID["mu1"] * (1 - a) + FLUID["mu2"] * a
        st = oracle.FluidState(n, 1.0 / n, taylor_green_cells(n), rho, mu, tol=FLUID["tol"])
        for s in range(1, max(steps) + 1):
            st.step(FLUID["dt"])
            if s not in steps:
                continue
            for name, v in (("vel", st.vel), ("p", st.p), ("flux", st.flux)):
                key = "%s%d_%d" % (name, q, s)
                assert np.array_equal(v[:8], fx[key + "_head"]), key
                assert hashlib.sha256(v.tobytes()).hexdigest() == str(fx[key]), key


def test_oracle_vof_source_equals_reference():
    """orc_vof_step_src (the volume source of Vof::MakeIteration,
    vof.ipp:504-514) equals aphros bit for bit after three steps."""
    fx = np.load(golden("vofsrc.npz"))
    n = int(fx["n"])
    case = workload.config("c1", n=n)
    st = oracle.VofState(n, case.h, case.alpha)
    for _ in range(int(fx["steps"])):
        st.step(case.flux, float(fx["dt"]), src=fx["src"])
    assert np.array_equal(st.u, fx["u_ref"])
    assert np.array_equal(st.nrm, fx["n_ref"], equal_nan=True)
    assert np.array_equal(st.a, fx["a_ref"], equal_nan=True)
    assert np.array_equal(st.curvature(), fx["k_ref"], equal_nan=True)


def _oracle_heights(n, h, u, nrm):
    st = oracle.VofState(n, h, u)
    st.nrm[:] = nrm
    return st.curvature()


@pytest.mark.parametrize("q", [0, 1])
def test_oracle_particle_curvature_equals_reference(q):
    """curvature::Particles and curvature::Hybrid with the part_* defaults
    (partcurv.npz: aphros's own estimators after VOF steps on one block,
    ref_harness REF_CURV): the oracle equals them bit for bit on the same
    PLIC state."""
    fx = np.load(golden("partcurv.npz"))
    n, h = int(fx["n%d" % q]), float(fx["h%d" % q])
    u, nrm, a = fx["u%d" % q], fx["nrm%d" % q], fx["a%d" % q]
    kp = oracle.curv_particles(n, h, u, nrm, a, nthreads=os.cpu_count() or 1)
    ref = fx["k_particles%d" % q]
    assert np.array_equal(np.isnan(kp), np.isnan(ref))
    m = ~np.isnan(ref)
    assert m.sum() > 500
    assert np.array_equal(kp[m], ref[m])
    kh = _oracle_heights(n, h, u, nrm)
    hyb = np.where(np.isnan(kh), kp, kh)
    ref = fx["k_hybrid%d" % q]
    assert np.array_equal(np.isnan(hyb), np.isnan(ref))
    m = ~np.isnan(ref)
    assert np.array_equal(hyb[m], ref[m])
    # the heights leave cells undefined that the particles fill
    assert (np.isnan(kh) & m).sum() > 10


def test_oracle_particle_curvature_sphere_and_parameters():
    """A sphere of radius 0.25 on 32^3: every interfacial cell gets a
    curvature, the mean is within 5 % of 2/R; parameters out of range are
    refused; fewer particles and strings change the estimate."""
    from aphros_gb300 import workload
    n = 32
    case = workload.Case(n, [(0.5, 0.5, 0.5)], [0.25], seed=1)
    st = oracle.VofState(n, case.h, case.alpha)
    st.reconstruct()
    k = oracle.curv_particles(n, case.h, st.u, st.nrm, st.a)
    ifc = (st.u > 0) & (st.u < 1)
    assert np.array_equal(~np.isnan(k), ifc)
    assert abs(np.mean(k[ifc]) - 8.0) < 0.4
    p = oracle.part_default()
    p.np = 6
    with pytest.raises(ValueError):
        oracle.curv_particles(n, case.h, st.u, st.nrm, st.a, par=p)
    p = oracle.part_default()
    p.np, p.ns = 5, 2
    k2 = oracle.curv_particles(n, case.h, st.u, st.nrm, st.a, par=p)
    assert np.array_equal(np.isnan(k2), np.isnan(k))
    assert not np.array_equal(k2[ifc], k[ifc])
