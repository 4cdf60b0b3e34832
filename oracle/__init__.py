"""CPU oracle (TEST INFRASTRUCTURE ONLY): ctypes binding of liboracle.so,
the plain-C restatement of aphros's projection-step hot path
(oracle/aphros_oracle.c).  Only tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py use it, always as the checker or the timed CPU
reference, never as part of the product path.

Parity of the oracle itself is pinned against aphros's own code compiled
from source (oracle/ref, `ref_harness`) and against the reference's golden
files: see tests/test_oracle_pins.py.
"""
import ctypes
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
REF_HARNESS = os.path.join(_HERE, "_ref", "ref_harness")

_D = ctypes.c_double
_P = ctypes.c_void_p
_PP3 = _P * 3
_I3 = ctypes.c_int * 3
_D3 = ctypes.c_double * 3


class OrcInfo(ctypes.Structure):
    _fields_ = [("residual", _D), ("iter", ctypes.c_int)]


_o = None


def lib():
    global _o
    if _o is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("liboracle.so not built: python -m aphros_gb300.build")
        o = ctypes.CDLL(LIB_PATH)
        o.orc_cg_solve.restype = OrcInfo
        o.orc_cg_solve.argtypes = [_I3, _D, _P, _P, _P, _D, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, _P, ctypes.c_int]
        o.orc_cg_time_iters.restype = _D
        o.orc_cg_time_iters.argtypes = [_I3, _P, _P, ctypes.c_int, ctypes.c_int]
        o.orc_residual.restype = _D
        o.orc_residual.argtypes = [_I3, _P, _P, _P]
        for name in ("orc_line_u", "orc_line_a"):
            getattr(o, name).restype = _D
        o.orc_line_u.argtypes = [_D3, _D, _D3]
        o.orc_line_a.argtypes = [_D3, _D, _D3]
        o.orc_line_flux.restype = _D
        o.orc_line_flux.argtypes = [_D3, _D, _D3, _D, _D, ctypes.c_int]
        o.orc_solve_cubic.restype = _D
        o.orc_solve_cubic.argtypes = [_D, _D, _D, _D, ctypes.c_int]
        o.orc_height_good.restype = _D
        o.orc_height_good.argtypes = [_P, ctypes.c_int]
        o.orc_height_good_n.restype = _D
        o.orc_fluid_step.restype = ctypes.c_int
        o.orc_height_good_n.argtypes = [_P, ctypes.c_int, _D]
        _o = o
    return _o


def _p(a):
    return None if a is None else a.ctypes.data_as(_P)


def _n3(n):
    n = (n, n, n) if isinstance(n, int) else tuple(n)
    return _I3(*n), n


def _faces(f, N):
    f = np.ascontiguousarray(f, dtype=np.float64)
    return f, _PP3(_p(f[:N]), _p(f[N:2 * N]), _p(f[2 * N:]))


def assemble_projection(n, h, dt, alpha, rho1, rho2, vflux, febp=None,
                        remove_mean=True):
    """Returns (expr8, k_faces, v_faces) as the reference assembles them."""
    o = lib()
    n3c, n3 = _n3(n)
    N = n3[0] * n3[1] * n3[2]
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    rho = np.empty(N)
    o.orc_mixture_density(ctypes.c_int64(N), _p(alpha), _D(rho1), _D(rho2), _p(rho))
    rf = np.empty(3 * N)
    rfa, rfp = _faces(rf, N)
    o.orc_face_density(n3c, _p(rho), rfp)
    vf, vfp = _faces(vflux, N)
    if febp is not None:
        fb, fbp = _faces(febp, N)
        vout = np.empty(3 * N)
        voa, vop = _faces(vout, N)
        o.orc_face_flux_with_force(n3c, _D(h), _D(dt), vfp, fbp, rfp, vop)
        vf, vfp = voa, vop
    e = np.empty(8 * N)
    fk = np.empty(3 * N)
    fka, fkp = _faces(fk, N)
    fv = np.empty(3 * N)
    fva, fvp = _faces(fv, N)
    o.orc_assemble_projection(n3c, _D(h), _D(dt), rfp, vfp, None, _p(e), fkp, fvp)
    if remove_mean:
        o.orc_remove_rhs_mean(ctypes.c_int64(N), _p(e))
    return e, fka, fva


def apply_cell_cond(expr8, cells, values):
    """Proj::ApplyCellCond (solver/proj.ipp:326-338): for each given-pressure
    cell c with value pc, e[0] += 1 and e[7] -= pc.  Returns a new array."""
    e = np.array(expr8, dtype=np.float64).reshape(-1, 8)
    for c, pc in zip(np.asarray(cells, dtype=np.int64), np.asarray(values, dtype=np.float64)):
        e[c, 0] += 1
        e[c, 7] -= pc
    return e.ravel()


def rel_tol(expr8, h, rtol=1e-10):
    """Absolute tolerance of the reference's CG norm sqrt(sum r^2/h^3) that
    corresponds to ||r||/||b|| = rtol with a zero guess (b = -e7)."""
    b = expr8[7::8]
    return rtol * math.sqrt(float(np.dot(b, b)) / h ** 3)


def cg_solve(n, h, expr8, tol, x0=None, miniter=1, maxiter=100000, maxnorm=0,
             nthreads=1, history=False):
    o = lib()
    n3c, n3 = _n3(n)
    N = n3[0] * n3[1] * n3[2]
    e = np.ascontiguousarray(expr8, dtype=np.float64)
    x = np.empty(N)
    x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
    hist = np.empty(maxiter + 2) if history else None
    info = o.orc_cg_solve(n3c, h ** 3, _p(e), _p(x0a), _p(x), tol, miniter, maxiter,
                          maxnorm, _p(hist), nthreads)
    if history:
        return x, info, hist[:info.iter]
    return x, info


def cg_time_iters(n, expr8, iters, nthreads=0):
    o = lib()
    n3c, n3 = _n3(n)
    N = n3[0] * n3[1] * n3[2]
    e = np.ascontiguousarray(expr8, dtype=np.float64)
    x = np.zeros(N)
    return o.orc_cg_time_iters(n3c, _p(e), _p(x), iters, nthreads)


def residual(n, expr8, x):
    o = lib()
    n3c, n3 = _n3(n)
    r = np.empty(n3[0] * n3[1] * n3[2])
    s = o.orc_residual(n3c, _p(np.ascontiguousarray(expr8)), _p(np.ascontiguousarray(x)), _p(r))
    return r, s


def flux_correct(n, fk, fv, p):
    o = lib()
    n3c, n3 = _n3(n)
    N = n3[0] * n3[1] * n3[2]
    _, fkp = _faces(fk, N)
    _, fvp = _faces(fv, N)
    out = np.empty(3 * N)
    oa, op = _faces(out, N)
    o.orc_flux_correct(n3c, fkp, fvp, _p(np.ascontiguousarray(p)), op)
    return oa


def acceleration(n, h, p, alpha, rho1, rho2, febp=None):
    o = lib()
    n3c, n3 = _n3(n)
    N = n3[0] * n3[1] * n3[2]
    rho = np.empty(N)
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    o.orc_mixture_density(ctypes.c_int64(N), _p(alpha), _D(rho1), _D(rho2), _p(rho))
    rf = np.empty(3 * N)
    _, rfp = _faces(rf, N)
    o.orc_face_density(n3c, _p(rho), rfp)
    fbp = None
    if febp is not None:
        _fb, fbp = _faces(febp, N)
    acc = np.empty(3 * N)
    o.orc_acceleration(n3c, _D(h), _p(np.ascontiguousarray(p)), rfp, fbp, _p(acc))
    return acc


def surface_tension(n, h, u, kappa, sigma):
    o = lib()
    n3c, n3 = _n3(n)
    N = n3[0] * n3[1] * n3[2]
    out = np.zeros(3 * N)
    oa, op = _faces(out, N)
    o.orc_surface_tension(n3c, _D(h), _p(np.ascontiguousarray(u)), _p(np.ascontiguousarray(kappa)),
                          _D(sigma), op)
    return oa


class VofState:
    """Vof state kept between steps (u, normals, plane constants, count)."""

    def __init__(self, n, h, u, clipth=1e-10):
        self.n3c, self.n3 = _n3(n)
        self.hh = _D3(h, h, h) if not hasattr(h, "__len__") else _D3(*h)
        N = self.n3[0] * self.n3[1] * self.n3[2]
        self.N = N
        self.u = np.array(u, dtype=np.float64)
        self.nrm = np.empty(3 * N)
        self.a = np.empty(N)
        self.mask = np.empty(N, dtype=np.uint8)
        self.clipth = clipth
        self.count = 0
        # colours as the reference's Vof starts them from a zero colour
        # field: 0 where u > 0, none (-1) elsewhere (vof.ipp:53-57)
        self.cl = np.where(self.u > 0, 0.0, -1.0)

    def step(self, vflux, dt, nthreads=1, src=None):
        """One MakeIteration; src: volume source per cell (None: zero)."""
        o = lib()
        if nthreads:
            os.environ.setdefault("OMP_NUM_THREADS", str(nthreads))
        vf, vfp = _faces(vflux, self.N)
        sa = None if src is None else np.ascontiguousarray(src, dtype=np.float64)
        o.orc_vof_step_src(self.n3c, self.hh, _p(self.u), vfp, _p(sa), _D(dt),
                           _D(self.clipth), self.count, 1 if self.count == 0 else 0,
                           self.mask.ctypes.data_as(_P), _p(self.nrm), _p(self.a))
        self.count += 1

    def reconstruct(self):
        """Vof::ReconstPlanes of the current field (mask, normals, plane
        constants), as the state after StartStep at t=0."""
        lib().orc_vof_reconstruct(self.n3c, self.hh, _p(self.u), self.mask.ctypes.data_as(_P),
                                  _p(self.nrm), _p(self.a))

    def recolor(self):
        """Connected-component colours of the current field (the resetcolor,
        union-find recolor and propagate stages of Vof::MakeIteration)."""
        out = np.empty(self.N)
        lib().orc_recolor(self.n3c, _p(self.u), _p(self.cl), _p(out))
        self.cl = out
        return out

    def curvature(self, heights=False):
        o = lib()
        k = np.empty(self.N)
        hg = np.empty(3 * self.N)
        o.orc_heights_curvature(self.n3c, self.hh, _p(self.u), _p(self.nrm), _p(k), _p(hg))
        return (k, hg) if heights else k


class PartPar(ctypes.Structure):
    """Parameters of the particle-string curvature (OrcPartPar)."""
    _fields_ = [("np", ctypes.c_int), ("ns", ctypes.c_int), ("leq", ctypes.c_double),
                ("relax", ctypes.c_double), ("tol", ctypes.c_double),
                ("itermax", ctypes.c_int), ("segcirc", ctypes.c_double), ("dn", ctypes.c_int)]


def part_default():
    """The part_* defaults of the reference's sim_base.conf."""
    p = PartPar()
    lib().orc_part_default(ctypes.byref(p))
    return p


def curv_particles(n, h, u, nrm, a, cl=None, par=None, nthreads=0):
    """curvature::Particles of the PLIC state (u, normals AoS, plane
    constants) with colours cl (None: no colours); NaN where no string is
    seeded (orc_curv_particles)."""
    n3c, n3 = _n3(n)
    N = n3[0] * n3[1] * n3[2]
    u = np.ascontiguousarray(u, dtype=np.float64)
    nrm = np.ascontiguousarray(nrm, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    cl = None if cl is None else np.ascontiguousarray(cl, dtype=np.float64)
    par = part_default() if par is None else par
    out = np.empty(N)
    o = lib()
    o.orc_curv_particles.restype = ctypes.c_int
    rc = o.orc_curv_particles(n3c, _D(h), _p(u), _p(nrm), _p(a), _p(cl), ctypes.byref(par),
                              _p(out), ctypes.c_int(nthreads))
    if rc != 0:
        raise ValueError("particle parameters out of range")
    return out


def recolor(n, u, cl_prev):
    """Colours of volume fraction u given the colours before (orc_recolor)."""
    n3c, n3 = _n3(n)
    u = np.ascontiguousarray(u, dtype=np.float64)
    cp = np.ascontiguousarray(cl_prev, dtype=np.float64)
    out = np.empty(n3[0] * n3[1] * n3[2])
    lib().orc_recolor(n3c, _p(u), _p(cp), _p(out))
    return out


class FluidState:
    """Proj (src/solver/proj.ipp) state between steps, periodic, default
    ProjPar, no forces: velocity (3 blocks), pressure, predictor pressure,
    face fluxes of the time layer."""

    def __init__(self, n, h, vel, rho, mu, tol=1e-8, maxiter=100000):
        self.n3c, self.n3 = _n3(n)
        N = self.n3[0] * self.n3[1] * self.n3[2]
        self.N, self.h = N, h
        self.vel = np.array(vel, dtype=np.float64)
        self.rho = np.ascontiguousarray(rho, dtype=np.float64)
        self.mu = np.ascontiguousarray(mu, dtype=np.float64)
        self.p = np.zeros(N)
        self.ppred = np.zeros(N)
        self.flux = np.empty(3 * N)
        self.tol, self.maxiter = tol, maxiter
        self.t_steps = 0
        fa, fp = _faces(self.flux, N)
        self.flux, self._fp = fa, fp
        lib().orc_fluid_init(self.n3c, _D(h), _p(self.vel), fp)

    def step(self, dt, nthreads=1):
        it = lib().orc_fluid_step(self.n3c, _D(self.h), _D(dt), _p(self.rho), _p(self.mu),
                                  _p(self.vel), _p(self.p), _p(self.ppred), self._fp,
                                  1 if self.t_steps == 0 else 0, _D(self.tol),
                                  ctypes.c_int(self.maxiter), ctypes.c_int(nthreads))
        self.t_steps += 1
        return it


def interpolate_bcg(n, h, u, vflux, src, dt):
    """Face values of the BCG predictor (orc_interpolate_bcg): 3 face blocks."""
    n3c, n3 = _n3(n)
    N = n3[0] * n3[1] * n3[2]
    u = np.ascontiguousarray(u, dtype=np.float64)
    s = np.ascontiguousarray(src, dtype=np.float64)
    vf, vfp = _faces(vflux, N)
    out = np.empty(3 * N)
    oa, op = _faces(out, N)
    lib().orc_interpolate_bcg(n3c, _D(h), _p(u), vfp, _p(s), _D(dt), op)
    return oa


def line_a(n, u, h):
    return lib().orc_line_a(_D3(*n), u, _D3(*h))


def line_u(n, a, h):
    return lib().orc_line_u(_D3(*n), a, _D3(*h))


def line_flux(n, a, h, q, dt, d):
    return lib().orc_line_flux(_D3(*n), a, _D3(*h), q, dt, d)


def height_good(uu):
    uu = np.ascontiguousarray(uu, dtype=np.float64)
    return lib().orc_height_good(_p(uu), len(uu))


def height_good_n(uu, nn):
    uu = np.ascontiguousarray(uu, dtype=np.float64)
    return lib().orc_height_good_n(_p(uu), len(uu), nn)
