"""ctypes binding of libaphgpu (include/aphgpu.h).

The CUDA library is the only implementation: if it is missing or cannot be
loaded this module raises, there is no fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libaphgpu.so")

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_NOMEM = 3
ERR_NOT_SYMMETRIC = 4
ERR_STATE = 5
ERR_UNSUPPORTED = 6
ERR_TIMEOUT = 7
OPT_GRAPHS = 0
OPT_FUSED_SWEEPS = 1
OPT_HALF_COUPLINGS = 2
OPT_CYCLE = 3
OPT_COARSE_SERIES = 4
OPT_SWEEP_GROWTH = 5
OPT_CTA_COARSE = 6
OPT_WAVE_PLANES = 7
OPT_COLOR_SPLIT = 8
OPT_DF_RESIDUAL = 9
OPT_W_MIN_CELLS = 10
FIELD_PRESSURE, FIELD_RHS, FIELD_VF, FIELD_CURVATURE = 0, 1, 2, 3
DUMP_UINT16, DUMP_FLOAT32, DUMP_FLOAT64 = 0, 1, 2

K_SMOOTH32, K_SMOOTH64, K_APPLY64, K_APPLY32, K_RESTRICT32 = 0, 1, 2, 3, 4
K_VOF_FLUX, K_VOF_UPDATE, K_RECONSTRUCT, K_HEIGHTS, K_CURVATURE = 5, 6, 7, 8, 9
K_SWEEP32 = 10
KERNEL_NAMES = {0: "KSmooth<float>", 1: "KSmooth<double>", 2: "KPcgApply<double>",
                3: "KPcgApply<float>", 4: "KResidualRestrict<float>",
                5: "KSweepFluxList", 6: "KSweepFused", 7: "KReconstruct",
                8: "KHeights", 9: "KCurvature", 10: "KSweepPipe"}

SOLVER_CG = 0
SOLVER_MGPCG = 1
SOLVER_MIXED = 2
SOLVER_MGPCG32 = 3

_D = ctypes.c_double
_I = ctypes.c_int
_P = ctypes.c_void_p
_PD = ctypes.POINTER(ctypes.c_double)


class Conf(ctypes.Structure):
    _fields_ = [
        ("solver", _I), ("tol", _D), ("miniter", _I), ("maxiter", _I),
        ("maxnorm", _I), ("mg_pre", _I), ("mg_post", _I),
        ("mg_coarse_max", _I), ("inner_rtol", _D), ("inner_maxiter", _I),
        ("inner_flags", _I), ("rtol", _D),
    ]


class Info(ctypes.Structure):
    _fields_ = [("residual", _D), ("iter", _I), ("inner_iter", _I),
                ("converged", _I)]


class PartConf(ctypes.Structure):
    """aphgpu_part_conf: parameters of the particle-string curvature."""
    _fields_ = [("np", ctypes.c_int), ("ns", ctypes.c_int), ("leq", ctypes.c_double),
                ("relax", ctypes.c_double), ("tol", ctypes.c_double),
                ("itermax", ctypes.c_int), ("segcirc", ctypes.c_double), ("dn", ctypes.c_int)]


CURV_HEIGHTS, CURV_PARTICLES, CURV_HYBRID = 0, 1, 2


class AphgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("aphgpu error %d: %s" % (code, msg))
        self.code = code


_lib = None


def lib():
    """Loads libaphgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libaphgpu.so not found at %s: build it with "
            "`python -m aphros_gb300.build`" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    L.aphgpu_conf_default.argtypes = [ctypes.POINTER(Conf)]
    L.aphgpu_conf_default.restype = None
    L.aphgpu_create.argtypes = [ctypes.POINTER(_P), _I, _I, _I, _D, _I]
    L.aphgpu_destroy.argtypes = [_P]
    L.aphgpu_destroy.restype = None
    L.aphgpu_last_error.argtypes = [_P]
    L.aphgpu_last_error.restype = ctypes.c_char_p
    L.aphgpu_device_bytes.argtypes = [_P]
    L.aphgpu_device_bytes.restype = ctypes.c_int64
    L.aphgpu_sync.argtypes = [_P]
    L.aphgpu_set_system_expr.argtypes = [_P, _P]
    L.aphgpu_get_system_expr.argtypes = [_P, _P]
    L.aphgpu_assemble_projection.argtypes = [_P, _P, _D, _D, _P, _P, _D, _I]
    L.aphgpu_solve.argtypes = [_P, ctypes.POINTER(Conf), _P, _P, ctypes.POINTER(Info)]
    L.aphgpu_solve_resident.argtypes = [_P, ctypes.POINTER(Conf), _I, ctypes.POINTER(Info)]
    L.aphgpu_get_solution.argtypes = [_P, _P]
    L.aphgpu_set_solution.argtypes = [_P, _P]
    L.aphgpu_set_solution.restype = _I
    L.aphgpu_residual_norms.argtypes = [_P, _PD, _PD]
    L.aphgpu_flux_correct.argtypes = [_P, _P]
    L.aphgpu_acceleration.argtypes = [_P, _P]
    L.aphgpu_vof_init.argtypes = [_P, _P, _D]
    L.aphgpu_vof_step.argtypes = [_P, _P, _D]
    L.aphgpu_vof_get.argtypes = [_P, _P, _P, _P, _P]
    L.aphgpu_fluid_init.argtypes = [_P, _P, _D, _D, _D, _D, _P]
    L.aphgpu_fluid_init.restype = _I
    L.aphgpu_fluid_step.argtypes = [_P, _D, ctypes.POINTER(Conf), ctypes.POINTER(Info)]
    L.aphgpu_fluid_step.restype = _I
    L.aphgpu_fluid_get.argtypes = [_P, _P, _P, _P]
    L.aphgpu_fluid_get.restype = _I
    L.aphgpu_bcg_faces.argtypes = [_P, _P, _P, _P, _D, _P]
    L.aphgpu_bcg_faces.restype = _I
    L.aphgpu_vof_set_source.argtypes = [_P, _P]
    L.aphgpu_vof_set_source.restype = _I
    L.aphgpu_apply_cell_cond.argtypes = [_P, ctypes.c_int64, _P, _P]
    L.aphgpu_apply_cell_cond.restype = _I
    L.aphgpu_curvature.argtypes = [_P, _P, _P]
    L.aphgpu_part_conf_default.argtypes = [ctypes.POINTER(PartConf)]
    L.aphgpu_part_conf_default.restype = None
    L.aphgpu_curvature_estimator.argtypes = [_P, _I, ctypes.POINTER(PartConf), _P]
    L.aphgpu_curvature_estimator.restype = _I
    L.aphgpu_surface_tension.argtypes = [_P, _D, _P]
    L.aphgpu_set_force_resident.argtypes = [_P, _I]
    L.aphgpu_last_timing.argtypes = [_P, _PD, ctypes.POINTER(ctypes.c_int64)]
    L.aphgpu_mark.argtypes = [_P, _I]
    L.aphgpu_set_option.argtypes = [_P, _I, _I]
    L.aphgpu_set_option.restype = _I
    L.aphgpu_vof_recolor.argtypes = [_P]
    L.aphgpu_vof_colors.argtypes = [_P, _P]
    L.aphgpu_dump_raw.argtypes = [_P, _I, _I, ctypes.c_char_p, ctypes.c_char_p]
    L.aphgpu_read_raw.argtypes = [_P, _I, ctypes.c_char_p, ctypes.c_char_p]
    L.aphgpu_xmf_text.argtypes = [_I, _I, _I, _D, ctypes.c_char_p, ctypes.c_char_p, _I,
                                  ctypes.c_char_p, _I, ctypes.POINTER(_I)]
    L.aphgpu_residual_history.argtypes = [_P, _I, _P, _I, ctypes.POINTER(_I)]
    L.aphgpu_residual_history.restype = _I
    L.aphgpu_elapsed.argtypes = [_P, _I, _I, _PD]
    L.aphgpu_time_kernel.argtypes = [_P, _I, _I, _PD, _PD]
    L.aphgpu_wave_wait_check.argtypes = [_P]
    L.aphgpu_batch_create.argtypes = [ctypes.POINTER(_P), _I, ctypes.POINTER(_P)]
    L.aphgpu_batch_destroy.argtypes = [_P]
    L.aphgpu_batch_destroy.restype = None
    L.aphgpu_batch_last_error.argtypes = [_P]
    L.aphgpu_batch_last_error.restype = ctypes.c_char_p
    L.aphgpu_batch_solve.argtypes = [_P, ctypes.POINTER(Conf), _P]
    L.aphgpu_batch_tune.argtypes = [_P, ctypes.POINTER(Conf), _PD]
    L.aphgpu_batch_last_ms.argtypes = [_P, _PD, ctypes.POINTER(ctypes.c_int64)]
    L.aphgpu_batch_set_tiles.argtypes = [_P, _I, _I]
    L.aphgpu_batch_get_tiles.argtypes = [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]
    L.aphgpu_batch_set_cycle.argtypes = [_P, _I]
    L.aphgpu_batch_get_cycle.argtypes = [_P, ctypes.POINTER(_I)]
    L.aphgpu_batch_set_cycle.restype = _I
    L.aphgpu_batch_get_cycle.restype = _I
    for name in ("aphgpu_batch_create", "aphgpu_batch_solve", "aphgpu_batch_tune",
                 "aphgpu_batch_last_ms", "aphgpu_batch_set_tiles", "aphgpu_batch_get_tiles"):
        getattr(L, name).restype = _I
    for name in ("aphgpu_create", "aphgpu_sync", "aphgpu_set_system_expr",
                 "aphgpu_get_system_expr",
                 "aphgpu_assemble_projection", "aphgpu_solve",
                 "aphgpu_solve_resident", "aphgpu_get_solution",
                 "aphgpu_residual_norms", "aphgpu_flux_correct",
                 "aphgpu_acceleration", "aphgpu_vof_init", "aphgpu_vof_step",
                 "aphgpu_vof_get", "aphgpu_curvature", "aphgpu_surface_tension",
                 "aphgpu_set_force_resident", "aphgpu_last_timing",
                 "aphgpu_mark", "aphgpu_elapsed", "aphgpu_time_kernel"):
        getattr(L, name).restype = _I
    _lib = L
    return L


def part_conf_default():
    """The reference's part_* defaults (aphgpu_part_conf_default)."""
    c = PartConf()
    lib().aphgpu_part_conf_default(ctypes.byref(c))
    return c


def ptr(a):
    """Pointer of a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(_P)


def default_conf(**kw):
    c = Conf()
    lib().aphgpu_conf_default(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def xmf_text(n, h, name, binpath, dtype=DUMP_FLOAT64):
    """The XMF metadata aphgpu_dump_raw writes (host only)."""
    n = (n, n, n) if isinstance(n, int) else tuple(n)
    L = lib()
    ln = _I()
    rc = L.aphgpu_xmf_text(n[0], n[1], n[2], h, name.encode(), binpath.encode(), dtype,
                           None, 0, ctypes.byref(ln))
    if rc != OK:
        raise AphgpuError(rc, "aphgpu_xmf_text failed")
    buf = ctypes.create_string_buffer(ln.value + 1)
    L.aphgpu_xmf_text(n[0], n[1], n[2], h, name.encode(), binpath.encode(), dtype,
                      buf, ln.value + 1, None)
    return buf.value.decode()


class Context:
    """One periodic nx*ny*nz domain resident on one GPU (aphgpu_ctx)."""

    def __init__(self, n, h, device=0):
        if isinstance(n, int):
            n = (n, n, n)
        self.n = tuple(int(v) for v in n)
        self.h = float(h)
        self.N = self.n[0] * self.n[1] * self.n[2]
        self._L = lib()
        p = _P()
        rc = self._L.aphgpu_create(ctypes.byref(p), self.n[0], self.n[1],
                                   self.n[2], self.h, device)
        if rc != OK:
            raise AphgpuError(rc, "aphgpu_create failed")
        self._p = p

    def close(self):
        if getattr(self, "_p", None):
            self._L.aphgpu_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._p

    def _check(self, rc):
        if rc != OK:
            msg = self._L.aphgpu_last_error(self._p)
            raise AphgpuError(rc, msg.decode() if msg else "")

    def _f64(self, a, count):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == count, "expected %d values, got %d" % (count, a.size)
        return a

    # ---- Poisson ----
    def set_system_expr(self, expr8):
        e = self._f64(expr8, 8 * self.N)
        self._check(self._L.aphgpu_set_system_expr(self._p, ptr(e)))

    def get_system_expr(self):
        e = np.empty(8 * self.N)
        self._check(self._L.aphgpu_get_system_expr(self._p, ptr(e)))
        return e

    def assemble_projection(self, alpha, rho1, rho2, vflux, dt, febp=None,
                            remove_mean=True):
        a = None if alpha is None else self._f64(alpha, self.N)
        v = self._f64(vflux, 3 * self.N)
        f = None if febp is None else self._f64(febp, 3 * self.N)
        self._check(self._L.aphgpu_assemble_projection(
            self._p, ptr(a), rho1, rho2, ptr(v), ptr(f), dt, int(remove_mean)))

    def solve(self, conf, x0=None, out=True):
        info = Info()
        x = np.empty(self.N) if out else None
        xi = None if x0 is None else self._f64(x0, self.N)
        self._check(self._L.aphgpu_solve(self._p, ctypes.byref(conf), ptr(xi),
                                         ptr(x), ctypes.byref(info)))
        return x, info

    def solve_resident(self, conf, zero_guess=True):
        info = Info()
        self._check(self._L.aphgpu_solve_resident(self._p, ctypes.byref(conf),
                                                  int(zero_guess), ctypes.byref(info)))
        return info

    def set_solution(self, x):
        a = self._f64(x, self.N)
        self._check(self._L.aphgpu_set_solution(self._p, ptr(a)))

    def get_solution(self):
        x = np.empty(self.N)
        self._check(self._L.aphgpu_get_solution(self._p, ptr(x)))
        return x

    def residual_norms(self):
        r, b = _D(), _D()
        self._check(self._L.aphgpu_residual_norms(self._p, ctypes.byref(r), ctypes.byref(b)))
        return r.value, b.value

    def flux_correct(self, out=True):
        v = np.empty(3 * self.N) if out else None
        self._check(self._L.aphgpu_flux_correct(self._p, ptr(v)))
        return v

    def acceleration(self):
        a = np.empty(3 * self.N)
        self._check(self._L.aphgpu_acceleration(self._p, ptr(a)))
        return a

    # ---- VOF ----
    def vof_init(self, alpha, clipth=1e-10):
        a = self._f64(alpha, self.N)
        self._check(self._L.aphgpu_vof_init(self._p, ptr(a), clipth))

    def vof_step(self, vflux, dt):
        v = None if vflux is None else self._f64(vflux, 3 * self.N)
        self._check(self._L.aphgpu_vof_step(self._p, ptr(v), dt))

    # ---- projection fluid step ----
    def fluid_init(self, alpha, rho1, rho2, mu1, mu2, vel):
        a = None if alpha is None else self._f64(alpha, self.N)
        v = self._f64(vel, 3 * self.N)
        self._check(self._L.aphgpu_fluid_init(self._p, ptr(a), rho1, rho2, mu1, mu2, ptr(v)))

    def fluid_step(self, dt, conf):
        info = Info()
        self._check(self._L.aphgpu_fluid_step(self._p, dt, ctypes.byref(conf),
                                              ctypes.byref(info)))
        return info

    def fluid_get(self):
        vel = np.empty(3 * self.N)
        p = np.empty(self.N)
        flux = np.empty(3 * self.N)
        self._check(self._L.aphgpu_fluid_get(self._p, ptr(vel), ptr(p), ptr(flux)))
        return vel, p, flux

    def bcg_faces(self, u, vflux, src, dt):
        out = np.empty(3 * self.N)
        self._check(self._L.aphgpu_bcg_faces(self._p, ptr(self._f64(u, self.N)),
                                             ptr(self._f64(vflux, 3 * self.N)),
                                             ptr(self._f64(src, self.N)), dt, ptr(out)))
        return out

    def vof_set_source(self, src):
        """Volume source of the following VOF steps (None: none)."""
        v = None if src is None else self._f64(src, self.N)
        self._check(self._L.aphgpu_vof_set_source(self._p, ptr(v)))

    def apply_cell_cond(self, cells, values):
        """Given-pressure cells of Proj::ApplyCellCond on the current system."""
        c = np.ascontiguousarray(cells, dtype=np.int64)
        v = np.ascontiguousarray(values, dtype=np.float64)
        if c.shape != v.shape:
            raise ValueError("cells and values differ in length")
        self._check(self._L.aphgpu_apply_cell_cond(self._p, len(c), ptr(c), ptr(v)))

    def vof_get(self):
        u = np.empty(self.N)
        nrm = np.empty(3 * self.N)
        a = np.empty(self.N)
        m = np.empty(self.N, dtype=np.uint8)
        self._check(self._L.aphgpu_vof_get(self._p, ptr(u), ptr(nrm), ptr(a), ptr(m)))
        return u, nrm, a, m

    def curvature_estimator(self, estimator, conf=None, out=True):
        """Curvature by the estimator (CURV_HEIGHTS, CURV_PARTICLES,
        CURV_HYBRID) with the particle parameters conf (None: defaults);
        out=False leaves it on the device (returns None)."""
        k = np.empty(self.N) if out else None
        pc = None if conf is None else ctypes.byref(conf)
        self._check(self._L.aphgpu_curvature_estimator(self._p, estimator, pc, ptr(k)))
        return k

    def curvature(self, heights=False, out=True):
        """Height-function curvature of the resident volume fraction; out=False
        leaves it on the device (returns None)."""
        k = np.empty(self.N) if out else None
        hg = np.empty(3 * self.N) if heights and out else None
        self._check(self._L.aphgpu_curvature(self._p, ptr(k), ptr(hg)))
        if not out:
            return None
        return (k, hg) if heights else k

    def surface_tension(self, sigma, out=True):
        f = np.empty(3 * self.N) if out else None
        self._check(self._L.aphgpu_surface_tension(self._p, sigma, ptr(f)))
        return f

    def set_force_resident(self, on=True):
        self._check(self._L.aphgpu_set_force_resident(self._p, int(on)))

    def last_timing(self):
        ms = _D()
        n = ctypes.c_int64()
        self._check(self._L.aphgpu_last_timing(self._p, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def residual_history(self, which=0):
        n = _I()
        self._check(self._L.aphgpu_residual_history(self._p, which, None, 0, ctypes.byref(n)))
        out = np.empty(n.value)
        self._check(self._L.aphgpu_residual_history(self._p, which, ptr(out), n.value,
                                                    ctypes.byref(n)))
        return out

    def set_option(self, option, value):
        """One of the OPT_* execution options (aphgpu_set_option)."""
        self._check(self._L.aphgpu_set_option(self._p, option, int(value)))

    def vof_recolor(self):
        """Connected-component colours of the current volume fraction."""
        self._check(self._L.aphgpu_vof_recolor(self._p))

    def vof_colors(self):
        cl = np.empty(self.N)
        self._check(self._L.aphgpu_vof_colors(self._p, ptr(cl)))
        return cl

    def dump_raw(self, field, rawpath, name, dtype=DUMP_FLOAT64):
        """Writes a field to rawpath and its XMF beside it (aphgpu_dump_raw)."""
        self._check(self._L.aphgpu_dump_raw(self._p, field, dtype, str(rawpath).encode(),
                                            name.encode()))

    def read_raw(self, field, xmfpath, rawpath=None):
        """Reads a field from a raw + XMF dump (aphgpu_read_raw)."""
        self._check(self._L.aphgpu_read_raw(
            self._p, field, str(xmfpath).encode(),
            None if rawpath is None else str(rawpath).encode()))

    def mark(self, slot):
        self._check(self._L.aphgpu_mark(self._p, slot))

    def elapsed(self, s0, s1):
        ms = _D()
        self._check(self._L.aphgpu_elapsed(self._p, s0, s1, ctypes.byref(ms)))
        return ms.value

    def time_kernel(self, kernel, reps=10):
        ms, b = _D(), _D()
        self._check(self._L.aphgpu_time_kernel(self._p, kernel, reps, ctypes.byref(ms),
                                               ctypes.byref(b)))
        return ms.value, b.value

    def device_bytes(self):
        return int(self._L.aphgpu_device_bytes(self._p))


class Batch:
    """Batched mixed-precision solve over many contexts (aphgpu_batch): one
    kernel launch per multigrid level covers every domain."""

    def __init__(self, ctxs):
        self._L = lib()
        self.ctxs = list(ctxs)
        arr = (_P * len(self.ctxs))(*[c.handle for c in self.ctxs])
        p = _P()
        rc = self._L.aphgpu_batch_create(ctypes.byref(p), len(self.ctxs), arr)
        if rc != OK:
            raise AphgpuError(rc, "aphgpu_batch_create failed")
        self._p = p

    def close(self):
        if getattr(self, "_p", None):
            self._L.aphgpu_batch_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != OK:
            msg = self._L.aphgpu_batch_last_error(self._p)
            raise AphgpuError(rc, msg.decode() if msg else "")

    def solve(self, conf):
        """Solves every domain; returns one Info per domain."""
        infos = (Info * len(self.ctxs))()
        self._check(self._L.aphgpu_batch_solve(self._p, ctypes.byref(conf),
                                               ctypes.cast(infos, _P)))
        return list(infos)

    def tune(self, conf):
        """Autotunes tiles and sweeps; updates conf and returns the best ms."""
        ms = _D()
        self._check(self._L.aphgpu_batch_tune(self._p, ctypes.byref(conf), ctypes.byref(ms)))
        return ms.value

    def set_tiles(self, planes, coarse_cells):
        self._check(self._L.aphgpu_batch_set_tiles(self._p, planes, coarse_cells))

    def tiles(self):
        """(z planes per tile, coarse-level cells of the per-domain cycle)."""
        a, b = _I(), _I()
        self._check(self._L.aphgpu_batch_get_tiles(self._p, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_cycle(self, cycle):
        self._check(self._L.aphgpu_batch_set_cycle(self._p, cycle))

    def cycle(self):
        v = _I()
        self._check(self._L.aphgpu_batch_get_cycle(self._p, ctypes.byref(v)))
        return v.value

    def last(self):
        ms, n = _D(), ctypes.c_int64()
        self._check(self._L.aphgpu_batch_last_ms(self._p, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, int(n.value)
