"""Synthetic inputs of the benchmarked configurations (libaphgen, host C).

Configurations (periodic unit cubes; gas volume fraction alpha = 1 inside
bubbles; liquid density rho1 = 1, gas rho2 = rho1 / ratio):
  c1   64^3, one sphere r=0.2 at the centre, ratio 1000, dt 1e-3
  c2   256^3, 16 spheres r in [0.03,0.08], seed 2
  c3   512^3, 64 spheres r in [0.02,0.05], seed 3
  c4   batch of domains, edge in {32,48,64,96}, 1-8 spheres of radius
       0.05-0.2 of the edge, ratio log-uniform in [10,1000], seed 4
  c5   served stream, edge 32-128 log-uniform rounded to a multiple of 16,
       1-8 bubbles, ratio 1000, seed 5
Predicted face fluxes: Taylor-Green (U=1) at face centres plus Gaussian
noise of standard deviation 0.01 per face, times the face area.
"""
import ctypes
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
GEN_PATH = os.path.join(_HERE, "_build", "libaphgen.so")
_D = ctypes.c_double
_P = ctypes.c_void_p
_g = None


def gen():
    global _g
    if _g is None:
        if not os.path.exists(GEN_PATH):
            raise ImportError("libaphgen.so not built: python -m aphros_gb300.build")
        g = ctypes.CDLL(GEN_PATH)
        g.aphgen_box_sphere.restype = _D
        g.aphgen_box_sphere.argtypes = [_D] * 7
        g.aphgen_alpha_spheres.argtypes = [ctypes.c_int] * 3 + [_D, ctypes.c_int, _P, _P, _P]
        g.aphgen_alpha_spheres.restype = None
        g.aphgen_place_spheres.argtypes = [ctypes.c_uint64, ctypes.c_int, _D, _D, _D, _P, _P]
        g.aphgen_place_spheres.restype = ctypes.c_int
        g.aphgen_tg_flux.argtypes = [ctypes.c_int] * 3 + [_D, _D, _D, ctypes.c_uint64, _P, _P, _P]
        g.aphgen_tg_flux.restype = None
        g.aphgen_uniform_flux.argtypes = [ctypes.c_int] * 3 + [_D] * 4 + [_P, _P, _P]
        g.aphgen_uniform_flux.restype = None
        g.aphgen_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        g.aphgen_uniform.restype = _D
        _g = g
    return _g


def _p(a):
    return a.ctypes.data_as(_P)


def alpha_spheres(n, centres, radii):
    """Gas volume fraction from exact sphere/cell overlap (periodic)."""
    n3 = (n, n, n) if isinstance(n, int) else tuple(n)
    h = 1.0 / max(n3)
    a = np.zeros(n3[0] * n3[1] * n3[2])
    c = np.ascontiguousarray(centres, dtype=np.float64).reshape(-1)
    r = np.ascontiguousarray(radii, dtype=np.float64).reshape(-1)
    gen().aphgen_alpha_spheres(n3[0], n3[1], n3[2], h, len(r), _p(c), _p(r), _p(a))
    return a


def place_spheres(seed, count, rmin, rmax, gap=None):
    if gap is None:
        gap = 0.5 * rmin
    c = np.zeros(3 * count)
    r = np.zeros(count)
    k = gen().aphgen_place_spheres(seed, count, rmin, rmax, gap, _p(c), _p(r))
    return c[:3 * k].reshape(k, 3), r[:k]


def tg_flux(n, U=1.0, noise=0.01, seed=1):
    """Face fluxes (3 blocks) of Taylor-Green plus noise."""
    n3 = (n, n, n) if isinstance(n, int) else tuple(n)
    h = 1.0 / max(n3)
    N = n3[0] * n3[1] * n3[2]
    f = np.empty(3 * N)
    gen().aphgen_tg_flux(n3[0], n3[1], n3[2], h, U, noise, seed,
                         _p(f[:N]), _p(f[N:2 * N]), _p(f[2 * N:]))
    return f


def uniform_flux(n3, h, vel):
    N = n3[0] * n3[1] * n3[2]
    f = np.empty(3 * N)
    gen().aphgen_uniform_flux(n3[0], n3[1], n3[2], h, vel[0], vel[1], vel[2],
                              _p(f[:N]), _p(f[N:2 * N]), _p(f[2 * N:]))
    return f


class Case:
    """One projection-step input: grid, bubbles, densities, fluxes."""

    def __init__(self, n, centres, radii, rho1=1.0, rho2=1e-3, dt=1e-3,
                 U=1.0, noise=0.01, seed=1):
        self.n = n
        self.h = 1.0 / n
        self.N = n ** 3
        self.centres = np.asarray(centres, dtype=np.float64).reshape(-1, 3)
        self.radii = np.asarray(radii, dtype=np.float64).reshape(-1)
        self.rho1, self.rho2, self.dt = rho1, rho2, dt
        self.U, self.noise, self.seed = U, noise, seed
        self._alpha = None
        self._flux = None

    @property
    def alpha(self):
        if self._alpha is None:
            self._alpha = alpha_spheres(self.n, self.centres, self.radii)
        return self._alpha

    @property
    def flux(self):
        if self._flux is None:
            self._flux = tg_flux(self.n, self.U, self.noise, self.seed)
        return self._flux

    def cfl_dt(self, cfl=0.5):
        """dt giving max |flux| / cell volume * dt = cfl."""
        mx = float(np.max(np.abs(self.flux))) / self.h ** 3
        return cfl / mx


def config(name, n=None):
    if name == "c1":
        return Case(n or 64, [[0.5, 0.5, 0.5]], [0.2], seed=1)
    if name == "c2":
        c, r = place_spheres(2, 16, 0.03, 0.08)
        return Case(n or 256, c, r, seed=2)
    if name == "c3":
        c, r = place_spheres(3, 64, 0.02, 0.05)
        return Case(n or 512, c, r, seed=3)
    raise ValueError(name)


def batch_cases(count, seed=4, edges=(32, 48, 64, 96)):
    """Batched configuration: independent domains of uneven size."""
    g = gen()
    out = []
    for i in range(count):
        u = lambda q: g.aphgen_uniform(seed, 16 * i + q)
        n = edges[min(int(u(0) * len(edges)), len(edges) - 1)]
        nb = 1 + min(int(u(1) * 8), 7)
        ratio = 10.0 ** (1 + 2 * u(2))
        c, r = place_spheres(seed * 100003 + i, nb, 0.05, 0.2, gap=0.02)
        out.append(Case(n, c, r, rho1=1.0, rho2=1.0 / ratio, seed=seed * 1000 + i))
    return out


def served_cases(count, seed=5, nmin=32, nmax=128, quantum=16):
    """Served configuration: edge log-uniform in [nmin,nmax] rounded to a
    multiple of `quantum`; with 16 every edge coarsens to a level of at most
    7^3 cells, solved by the dense coarsest inverse."""
    g = gen()
    out = []
    for i in range(count):
        u = lambda q: g.aphgen_uniform(seed, 16 * i + q)
        e = math.exp(math.log(nmin) + (math.log(nmax) - math.log(nmin)) * u(0))
        n = int(max(nmin, min(nmax, quantum * round(e / quantum))))
        nb = 1 + min(int(u(1) * 8), 7)
        c, r = place_spheres(seed * 100003 + i, nb, 0.05, 0.15, gap=0.02)
        out.append(Case(n, c, r, rho1=1.0, rho2=1e-3, seed=seed * 1000 + i))
    return out
