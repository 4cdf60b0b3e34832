"""Generates the golden fixtures of tests/golden/ by running aphros's OWN code
(oracle/_ref/ref_harness, built from the reference sources by
oracle/ref/Makefile) and by reading the reference's committed test data.

Run from the repository root, where the reference tree is available:
    python tests/golden/make_golden.py [--ref /path/to/aphros]

Fixtures:
  advection3d.npz  the reference's 3-D advection test (test/advection,
                   24x24x16, uniform velocity (0.6,0.5,0.3), Weymouth):
                   initial field and golden result from its ref/3d/*.dat, and
                   aphros's own run of the 58 steps on one block (u, normals,
                   plane constants, curvature).
  proj16.npz       projection step on 16^3 (sphere r=0.2, density ratio
                   1000, Taylor-Green + noise): inputs, aphros's assembled
                   system, CG solution at ||r||/||b|| = 1e-10, corrected
                   fluxes, iteration count.
  proj64.npz       C1 projection system on 64^3 (sphere r=0.2, density
                   ratio 1000, Taylor-Green + noise, from the workload
                   generator; SHA-256 of the inputs stored): aphros's CG
                   solution at ||r||/||b|| = 1e-13 (blocks of 16^3, all
                   host threads), its residual and iteration count.
  vof32.npz        3 VOF steps + Heights curvature on 32^3 (sphere r=0.2,
                   Taylor-Green flux at CFL 0.5): aphros's results.
  vofsrc.npz       3 VOF steps on 32^3 (sphere r=0.2, Taylor-Green flux at
                   CFL 0.5) with a volume source (Vof's fcs, vof.ipp:510-513)
                   that vanishes within two cells of the block boundary:
                   aphros's results (u, normals, plane constants, curvature).
  reconst.txt      random planes: GetLineA, GetLineU, GetLineFlux.
  height.txt       UHeight::Good on the reference's unit-test columns
                   (test/util/main.cpp) and on random 13-cell columns.
  overlap.txt      GetSphereOverlap on random boxes (pins the generator).
  colors.npz       Vof::GetColor (union-find recolouring) after 1, 3 and 8
                   steps on one 32^3 block: 8 separate bubbles, 10 bubbles
                   some of which touch, and spheres across the periodic
                   boundary with a touching pair (inputs from the workload
                   generator, stored as parameters).
  fluid.npz        the projection fluid solver Proj (default ProjPar: BCG,
                   implicit diffusion) run by aphros for 1 and 4 steps on a
                   12^3 sphere and a 16^3 four-bubble field (density ratio
                   1000, Taylor-Green start): SHA-256 digests of the
                   velocity, pressure and face fluxes, and a few values.
  bcg.npz          UEmbed::InterpolateBcg face values on periodic 12x10x8
                   and 8^3 meshes (random cell field, face fluxes and
                   source).
  partcurv.npz     curvature::Particles and curvature::Hybrid (part_*
                   defaults of sim_base.conf) after 3 VOF steps on one 32^3
                   block (C1 sphere, Taylor-Green flux at CFL 0.5) and after
                   2 steps on one 48^3 block of 16 bubbles (C2 draw): the
                   PLIC state (u, normals, plane constants) and both
                   curvature fields.
  dumps.npz        dump::Xmf::WriteXmf texts of dump::Raw::WriteWithXmf
                   metadata for several meshes and element types, and
                   dump::Raw::WriteBlocks output of a 3x4x5 array converted
                   to Double, Float and UShort.
"""
import argparse
import math
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from aphros_gb300 import workload  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def read_plain(path):
    with open(path) as f:
        dims = [int(v) for v in f.readline().split()]
        data = np.array(f.read().split(), dtype=float)
    return dims, data


def run(args, cwd, threads=1):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    subprocess.run([HARNESS] + args, cwd=cwd, check=True, env=env)


def advection3d(ref, tmp):
    d = os.path.join(ref, "src", "test", "advection", "ref", "3d")
    dims, u0 = read_plain(os.path.join(d, "u_0000.dat"))
    _, u2 = read_plain(os.path.join(d, "u_0002.dat"))
    n3 = tuple(dims)
    h = 1.0 / max(n3)
    vel = (0.6, 0.5, 0.3)
    flux = workload.uniform_flux(n3, h, vel)
    # dt = cfl / maxvel with cfl 0.25 (test/advection/std.conf, main.cpp:234-241)
    area, vol = h * h, h * h * h
    maxvel = max(abs(flux[:]).max() / vol, 0.0)
    dt = float(0.25 / maxvel)
    steps = 58  # first dump time >= tmax with dump_field_dt 0.5, tmax 1
    u0.tofile(os.path.join(tmp, "u0.bin"))
    flux.tofile(os.path.join(tmp, "f.bin"))
    run(["vof", "%d,%d,%d" % n3, "%d,%d,%d" % n3, repr(h), repr(dt), str(steps),
         "u0.bin", "f.bin", "adv"], tmp)
    r = lambda s: np.fromfile(os.path.join(tmp, "adv." + s))
    np.savez_compressed(os.path.join(OUT, "advection3d.npz"), n=np.array(n3), h=h,
                        dt=dt, steps=steps, vel=np.array(vel), u_init=u0,
                        u_golden=u2, u_ref=r("u"), n_ref=r("n"), a_ref=r("a"),
                        k_ref=r("k"))


def proj16(tmp):
    case = workload.config("c1", n=16)
    n, h = case.n, case.h
    case.alpha.tofile(os.path.join(tmp, "alpha.bin"))
    case.flux.tofile(os.path.join(tmp, "vf.bin"))
    # tolerance for ||r||/||b|| = 1e-10 in the reference's norm
    import oracle
    e, _, _ = oracle.assemble_projection(n, h, case.dt, case.alpha, case.rho1,
                                         case.rho2, case.flux)
    tol = oracle.rel_tol(e, h, 1e-10)
    run(["proj", str(n), str(n), repr(h), repr(case.dt), repr(case.rho1),
         repr(case.rho2), repr(tol), "100000", "alpha.bin", "vf.bin", "pr"], tmp)
    r = lambda s: np.fromfile(os.path.join(tmp, "pr." + s))
    info = open(os.path.join(tmp, "pr.info")).read().split()
    expr_ref, p_ref, flux_ref = r("expr"), r("p"), r("flux")
    # the same solve on 8 blocks of 8^3: the reference's own spread due to
    # the order of its reductions
    run(["proj", str(n), "8", repr(h), repr(case.dt), repr(case.rho1),
         repr(case.rho2), repr(tol), "100000", "alpha.bin", "vf.bin", "pr8"], tmp)
    info8 = open(os.path.join(tmp, "pr8.info")).read().split()
    p8 = np.fromfile(os.path.join(tmp, "pr8.p"))
    np.savez_compressed(os.path.join(OUT, "proj16.npz"), n=n, h=h, dt=case.dt,
                        rho1=case.rho1, rho2=case.rho2, tol=tol, alpha=case.alpha,
                        vflux=case.flux, expr_ref=expr_ref, p_ref=p_ref,
                        flux_ref=flux_ref, residual=float(info[0]),
                        iters=int(info[1]), iters_blocks8=int(info8[1]),
                        p_blocks8=p8)


def proj64(tmp):
    import hashlib

    import oracle
    case = workload.config("c1", n=64)
    n, h = case.n, case.h
    case.alpha.tofile(os.path.join(tmp, "alpha.bin"))
    case.flux.tofile(os.path.join(tmp, "vf.bin"))
    e, _, _ = oracle.assemble_projection(n, h, case.dt, case.alpha, case.rho1,
                                         case.rho2, case.flux)
    tol = oracle.rel_tol(e, h, 1e-13)
    run(["proj", str(n), "16", repr(h), repr(case.dt), repr(case.rho1),
         repr(case.rho2), repr(tol), "1000000", "alpha.bin", "vf.bin", "p64"], tmp,
        threads=os.cpu_count() or 1)
    info = open(os.path.join(tmp, "p64.info")).read().split()
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    np.savez_compressed(os.path.join(OUT, "proj64.npz"), n=n, h=h, dt=case.dt,
                        rho1=case.rho1, rho2=case.rho2, tol=tol, rtol=1e-13,
                        alpha_sha256=sha(case.alpha), flux_sha256=sha(case.flux),
                        p_ref=np.fromfile(os.path.join(tmp, "p64.p")),
                        residual=float(info[0]), iters=int(info[1]))


def vof32(tmp):
    case = workload.config("c1", n=32)
    n, h = case.n, case.h
    dt = case.cfl_dt(0.5)
    case.alpha.tofile(os.path.join(tmp, "a.bin"))
    case.flux.tofile(os.path.join(tmp, "f.bin"))
    run(["vof", str(n), str(n), repr(h), repr(dt), "3", "a.bin", "f.bin", "v"], tmp)
    r = lambda s: np.fromfile(os.path.join(tmp, "v." + s))
    np.savez_compressed(os.path.join(OUT, "vof32.npz"), n=n, h=h, dt=dt, steps=3,
                        u_ref=r("u"), n_ref=r("n"), a_ref=r("a"), k_ref=r("k"),
                        alpha_sum=float(case.alpha.sum()))


def vof_source(n, seed=11):
    """Volume source of the vofsrc fixture: half-integer multiples of 0.5 in
    [-6, 6], zero within two cells of the boundary (there the reference's
    first sweep would read halo values from before the source)."""
    rng = np.random.default_rng(seed)
    s = np.clip(np.round(rng.normal(size=(n, n, n)) * 4) / 2, -6, 6)
    inner = np.zeros((n, n, n), bool)
    inner[2:n - 2, 2:n - 2, 2:n - 2] = True
    return np.where(inner, s, 0.0).ravel()


def vofsrc(tmp):
    case = workload.config("c1", n=32)
    n, h = case.n, case.h
    dt = case.cfl_dt(0.5)
    src = vof_source(n)
    case.alpha.tofile(os.path.join(tmp, "a.bin"))
    case.flux.tofile(os.path.join(tmp, "f.bin"))
    src.tofile(os.path.join(tmp, "s.bin"))
    os.environ["REF_VOF_SRC"] = os.path.join(tmp, "s.bin")
    try:
        run(["vof", str(n), str(n), repr(h), repr(dt), "3", "a.bin", "f.bin", "vs"], tmp)
    finally:
        del os.environ["REF_VOF_SRC"]
    r = lambda q: np.fromfile(os.path.join(tmp, "vs." + q))
    np.savez_compressed(os.path.join(OUT, "vofsrc.npz"), n=n, h=h, dt=dt, steps=3,
                        src=src, u_ref=r("u"), n_ref=r("n"), a_ref=r("a"), k_ref=r("k"))


def partcurv(tmp):
    out = {}
    for q, (cname, n, steps) in enumerate((("c1", 32, 3), ("c2", 48, 2))):
        case = workload.config(cname, n=n)
        dt = case.cfl_dt(0.5)
        case.alpha.tofile(os.path.join(tmp, "a.bin"))
        case.flux.tofile(os.path.join(tmp, "f.bin"))
        for est in ("particles", "hybrid"):
            os.environ["REF_CURV"] = est
            try:
                run(["vof", str(n), str(n), repr(case.h), repr(dt), str(steps), "a.bin",
                     "f.bin", "pc"], tmp)
            finally:
                del os.environ["REF_CURV"]
            r = lambda s_: np.fromfile(os.path.join(tmp, "pc." + s_))
            out["k_%s%d" % (est, q)] = r("k")
        out.update({"n%d" % q: n, "h%d" % q: case.h, "dt%d" % q: dt, "steps%d" % q: steps,
                    "case%d" % q: cname, "u%d" % q: r("u"), "nrm%d" % q: r("n"),
                    "a%d" % q: r("a")})
    np.savez_compressed(os.path.join(OUT, "partcurv.npz"), **out)


def reconst(tmp, rows=300):
    rng = np.random.default_rng(7)
    lines = []
    for i in range(rows):
        n = rng.normal(size=3)
        if i % 5 == 0:
            n[rng.integers(3)] = 0.0
        if i % 11 == 0:
            n[:] = 0
            n[rng.integers(3)] = 1.0
        n /= np.abs(n).sum()
        h = rng.uniform(0.5, 2.0, size=3) if i % 3 == 0 else np.full(3, 1.0 / 32)
        u = rng.uniform(0, 1)
        if i % 7 == 0:
            u = rng.choice([1e-9, 0.5, 1 - 1e-9])
        a = rng.uniform(-0.5, 0.5) * np.abs(n * h).sum()
        d = int(rng.integers(3))
        area = h.prod() / h[d]
        dt = 0.01
        q = rng.uniform(-0.9, 0.9) * h[d] * area / dt
        lines.append(" ".join(repr(float(v)) for v in
                              [*n, u, a, *h, q, dt, d]))
    src = os.path.join(tmp, "rin.txt")
    open(src, "w").write("\n".join(lines) + "\n")
    run(["reconst", "rin.txt", "rout.txt"], tmp)
    out = open(os.path.join(tmp, "rout.txt")).read().split("\n")
    with open(os.path.join(OUT, "reconst.txt"), "w") as f:
        f.write("# n0 n1 n2 u a h0 h1 h2 q dt d | GetLineA(n,u,h) GetLineU(n,a,h) "
                "GetLineFlux(n,a,h,q,dt,d) from aphros (src/solver/reconst.h)\n")
        for a, b in zip(lines, out):
            f.write(a + " | " + b + "\n")


def height(ref, tmp, rows=300):
    src = open(os.path.join(ref, "src", "test", "util", "main.cpp")).read()
    cols = []
    # t({...}, n, bool) in TestGood and t({...}, value) in TestGood2
    for m in re.finditer(r"t\(\{([^}]*)\},\s*([-\w.]+)\s*(?:,\s*(true|false))?\)", src):
        vals = [float(v) for v in m.group(1).split(",")]
        if m.group(3) is not None:
            cols.append((vals, float(m.group(2)), m.group(3)))
        else:
            cols.append((vals, None, m.group(2)))
    rng = np.random.default_rng(11)
    for i in range(rows):
        c = np.where(rng.uniform(size=13) < 0.5, 0.0, 1.0)
        k = int(rng.integers(2, 11))
        c[k - 2:k + 3] = np.sort(rng.uniform(size=5))[:: (1 if i % 2 else -1)]
        c[6] = rng.uniform(0.05, 0.95)
        cols.append(([float(v) for v in c], None, "random"))
    lines = []
    for vals, nn, _ in cols:
        lines.append(("n=%r " % nn if nn is not None else "") +
                     " ".join(repr(v) for v in vals))
    open(os.path.join(tmp, "hin.txt"), "w").write("\n".join(lines) + "\n")
    run(["height", "hin.txt", "hout.txt"], tmp)
    out = open(os.path.join(tmp, "hout.txt")).read().split("\n")
    with open(os.path.join(OUT, "height.txt"), "w") as f:
        f.write("# column (n=<normal> for the two-argument form) | UHeight::Good "
                "from aphros (src/util/height.h) | expectation of "
                "test/util/main.cpp or 'random'\n")
        for (vals, nn, exp), line, res in zip(cols, lines, out):
            f.write(line + " | " + res + " | " + exp + "\n")


def overlap(tmp, rows=200):
    rng = np.random.default_rng(13)
    lines = []
    for i in range(rows):
        r = rng.uniform(0.05, 0.3)
        c = rng.uniform(0.2, 0.8, size=3)
        h = np.full(3, rng.choice([1 / 16, 1 / 32, 1 / 64]))
        # box centres near the sphere surface
        dirn = rng.normal(size=3)
        dirn /= np.linalg.norm(dirn)
        x = c + dirn * (r + rng.uniform(-1.5, 1.5) * h[0])
        lines.append(" ".join(repr(float(v)) for v in [*x, *h, *c, r]))
    open(os.path.join(tmp, "oin.txt"), "w").write("\n".join(lines) + "\n")
    run(["overlap", "oin.txt", "oout.txt"], tmp)
    out = open(os.path.join(tmp, "oout.txt")).read().split("\n")
    with open(os.path.join(OUT, "overlap.txt"), "w") as f:
        f.write("# x y z hx hy hz cx cy cz r | GetSphereOverlap from aphros "
                "(src/overlap/overlap.h)\n")
        for a, b in zip(lines, out):
            f.write(a + " | " + b + "\n")


def bcg(tmp):
    rng = np.random.default_rng(5)
    out = {}
    for q, n3 in enumerate(((12, 10, 8), (8, 8, 8))):
        N = n3[0] * n3[1] * n3[2]
        h = 1.0 / max(n3)
        u = rng.normal(size=N)
        vf = rng.normal(size=3 * N) * h * h
        src = rng.normal(size=N)
        dt = 0.01
        u.tofile(os.path.join(tmp, "bu.bin"))
        vf.tofile(os.path.join(tmp, "bv.bin"))
        src.tofile(os.path.join(tmp, "bs.bin"))
        ns = "%d,%d,%d" % n3
        run(["bcg", ns, ns, repr(dt), "bu.bin", "bv.bin", "bs.bin", "bo"], tmp)
        out.update({"n%d" % q: np.array(n3), "h%d" % q: h, "dt%d" % q: dt, "u%d" % q: u,
                    "vflux%d" % q: vf, "src%d" % q: src,
                    "ffu%d" % q: np.fromfile(os.path.join(tmp, "bo.ffu"))})
    np.savez_compressed(os.path.join(OUT, "bcg.npz"), **out)


FLUID = dict(rho1=1.0, rho2=0.001, mu1=0.01, mu2=0.0001, dt=0.002, tol=1e-8)
FLUID_STEPS = (1, 4)


def taylor_green_cells(n):
    """Cell velocity (3 blocks) of the Taylor-Green vortex, periodic unit cube."""
    h = 1.0 / n
    k, j, i = np.indices((n, n, n))
    x, y, z = (i + 0.5) * h, (j + 0.5) * h, (k + 0.5) * h
    vx = np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y) * np.cos(2 * np.pi * z)
    vy = -np.cos(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.cos(2 * np.pi * z)
    return np.concatenate([vx.ravel(), vy.ravel(), np.zeros(n ** 3)])


def fluid_cases():
    c, r = workload.place_spheres(9, 4, 0.1, 0.18, gap=0.03)
    return [(12, np.array([[0.5, 0.5, 0.5]]), np.array([0.2])), (16, c, r)]


def fluid(tmp):
    import hashlib
    out = {"steps": np.array(FLUID_STEPS)}
    for q, (n, c, r) in enumerate(fluid_cases()):
        case = workload.Case(n, c, r, seed=1)
        case.alpha.tofile(os.path.join(tmp, "fa.bin"))
        taylor_green_cells(n).tofile(os.path.join(tmp, "fv.bin"))
        out["n%d" % q] = n
        out["centres%d" % q] = np.asarray(c)
        out["radii%d" % q] = np.asarray(r)
        for s in FLUID_STEPS:
            f = FLUID
            run(["fluid", str(n), str(n), repr(f["dt"]), str(s), repr(f["rho1"]), repr(f["rho2"]),
                 repr(f["mu1"]), repr(f["mu2"]), repr(f["tol"]), "100000", "fa.bin", "fv.bin",
                 "fo"], tmp)
            for name in ("vel", "p", "flux"):
                a = np.fromfile(os.path.join(tmp, "fo." + name))
                out["%s%d_%d" % (name, q, s)] = np.array(hashlib.sha256(a.tobytes()).hexdigest())
                out["%s%d_%d_head" % (name, q, s)] = a[:8]
    np.savez(os.path.join(OUT, "fluid.npz"), **out)


COLOR_STEPS = (1, 3, 8)


def color_cases():
    """(name, n, centres, radii, flux seed) of the colour fixtures."""
    c0, r0 = workload.place_spheres(31, 8, 0.06, 0.14, gap=0.03)
    c1, r1 = workload.place_spheres(77, 10, 0.08, 0.16, gap=0.0)
    c2 = np.array([[0.02, 0.5, 0.5], [0.5, 0.97, 0.03], [0.5, 0.5, 0.5], [0.62, 0.5, 0.5]])
    r2 = np.array([0.12, 0.1, 0.07, 0.07])
    return [("separate", 32, c0, r0, 32), ("touching", 32, c1, r1, 9),
            ("periodic", 32, c2, r2, 9)]


def colors(tmp):
    out = {"steps": np.array(COLOR_STEPS)}
    for q, (name, n, c, r, seed) in enumerate(color_cases()):
        case = workload.Case(n, c, r, seed=seed)
        dt = case.cfl_dt(0.5)
        case.alpha.tofile(os.path.join(tmp, "ca.bin"))
        case.flux.tofile(os.path.join(tmp, "cf.bin"))
        out["n%d" % q] = n
        out["centres%d" % q] = np.asarray(c)
        out["radii%d" % q] = np.asarray(r)
        out["seed%d" % q] = seed
        for s in COLOR_STEPS:
            run(["vof", str(n), str(n), repr(case.h), repr(dt), str(s), "ca.bin", "cf.bin",
                 "cv"], tmp)
            cl = np.fromfile(os.path.join(tmp, "cv.cl"))
            assert np.all(cl == np.round(cl)) and cl.min() >= -1 and cl.max() < 32767
            out["cl%d_%d" % (q, s)] = cl.astype(np.int16)
    np.savez_compressed(os.path.join(OUT, "colors.npz"), **out)


XMF_CASES = [  # (nx, ny, nz, h, name, binpath, type)
    (16, 16, 16, 1 / 16, "vf", "vf.raw", "Double"),
    (32, 24, 16, 1 / 32, "p", "out/p_0001.raw", "Float"),
    (8, 8, 8, 0.125, "cl", "cl.raw", "UShort"),
    (48, 48, 48, 1 / 48, "kappa", "/tmp/k.raw", "Double"),
]


def dumps(tmp):
    out = {}
    for q, (nx, ny, nz, h, name, binpath, typ) in enumerate(XMF_CASES):
        path = os.path.join(tmp, "x%d.xmf" % q)
        run(["xmf", "%d,%d,%d" % (nx, ny, nz), repr(h), name, binpath, typ, path], tmp)
        out["xmf%d" % q] = np.array(open(path).read())
    # a 3x4x5 array: fractions, values that round differently in float32,
    # and values whose truncation to uint16 is exact
    rng = np.random.default_rng(17)
    v = rng.uniform(0, 60000, size=60) + rng.uniform(0, 1, size=60) / 3
    v[:4] = [0.0, 1.5, 65535.25, 1 / 3]
    v.astype(np.float64).tofile(os.path.join(tmp, "v.f64"))
    out["values"] = v
    for typ in ("Double", "Float", "UShort"):
        path = os.path.join(tmp, "v_%s.raw" % typ)
        run(["raw", "3,4,5", typ, "v.f64", path], tmp)
        out["raw_" + typ] = np.fromfile(path, dtype=np.uint8)
    np.savez(os.path.join(OUT, "dumps.npz"), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.path.join(ROOT, "baseline", "_ref", "aphros"))
    ap.add_argument("--only", default="", help="comma-separated fixture names")
    args = ap.parse_args()
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: python -m aphros_gb300.build")
    makers = [("advection3d", lambda t: advection3d(args.ref, t)), ("proj16", proj16),
              ("proj64", proj64), ("vof32", vof32), ("vofsrc", vofsrc), ("reconst", reconst),
              ("height", lambda t: height(args.ref, t)), ("overlap", overlap),
              ("dumps", dumps), ("colors", colors), ("bcg", bcg), ("fluid", fluid),
              ("partcurv", partcurv)]
    only = set(filter(None, args.only.split(",")))
    with tempfile.TemporaryDirectory() as tmp:
        for name, make in makers:
            if not only or name in only:
                make(tmp)
    for f in sorted(os.listdir(OUT)):
        print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
