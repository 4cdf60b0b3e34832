"""Serving loop binding (aphgpu_server_* of include/aphgpu.h).

    srv = Server(budget_bytes=150e9, slots=8)
    sim = srv.add(case)                  # workload.Case: grid, bubbles, densities
    t = srv.submit(sim, vflux, dt)       # one full step, returns a ticket
    res = srv.wait(t)                    # latency, iterations, status
"""
import ctypes

import numpy as np

from . import _lib

_I64 = ctypes.c_int64


class StepResult(ctypes.Structure):
    _fields_ = [("ticket", _I64), ("sim", ctypes.c_int), ("status", ctypes.c_int),
                ("iters", ctypes.c_int), ("inner_iters", ctypes.c_int),
                ("converged", ctypes.c_int), ("residual", ctypes.c_double),
                ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("device_ms", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("sims", ctypes.c_int), ("resident", ctypes.c_int),
                ("resident_bytes", _I64), ("budget_bytes", _I64), ("completed", _I64),
                ("queued", _I64), ("evictions", _I64), ("admissions", _I64)]


def _bind():
    L = _lib.lib()
    P = ctypes.c_void_p
    L.aphgpu_server_create.argtypes = [ctypes.POINTER(P), ctypes.c_int, ctypes.c_double,
                                       ctypes.c_int, ctypes.POINTER(_lib.Conf)]
    L.aphgpu_server_destroy.argtypes = [P]
    L.aphgpu_server_destroy.restype = None
    L.aphgpu_server_add_sim.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, P, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
    L.aphgpu_server_submit.argtypes = [P, ctypes.c_int, P, ctypes.c_double,
                                       ctypes.POINTER(_I64)]
    L.aphgpu_server_wait.argtypes = [P, _I64, ctypes.POINTER(StepResult)]
    L.aphgpu_server_wait_timeout.argtypes = [P, _I64, ctypes.c_double,
                                             ctypes.POINTER(StepResult)]
    L.aphgpu_server_get_state.argtypes = [P, ctypes.c_int, P, P]
    L.aphgpu_server_get_stats.argtypes = [P, ctypes.POINTER(Stats)]
    for n in ("aphgpu_server_create", "aphgpu_server_add_sim", "aphgpu_server_submit",
              "aphgpu_server_wait", "aphgpu_server_wait_timeout", "aphgpu_server_get_state",
              "aphgpu_server_get_stats"):
        getattr(L, n).restype = ctypes.c_int
    return L


class Server:
    def __init__(self, budget_bytes=150e9, slots=8, conf=None, device=0):
        self._L = _bind()
        p = ctypes.c_void_p()
        c = None if conf is None else ctypes.byref(conf)
        rc = self._L.aphgpu_server_create(ctypes.byref(p), device, float(budget_bytes),
                                          slots, c)
        if rc != _lib.OK:
            raise _lib.AphgpuError(rc, "aphgpu_server_create failed")
        self._p = p
        self.sizes = {}

    def close(self):
        if getattr(self, "_p", None):
            self._L.aphgpu_server_destroy(self._p)
            self._p = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc != _lib.OK:
            raise _lib.AphgpuError(rc, what)

    def add(self, case, sigma=0.0):
        sim = ctypes.c_int()
        a = np.ascontiguousarray(case.alpha, dtype=np.float64)
        self._check(self._L.aphgpu_server_add_sim(self._p, case.n, case.n, case.n, case.h,
                                                  _lib.ptr(a), case.rho1, case.rho2, sigma,
                                                  ctypes.byref(sim)), "add_sim")
        self.sizes[sim.value] = case.N
        return sim.value

    def submit(self, sim, vflux, dt):
        v = np.ascontiguousarray(vflux, dtype=np.float64)
        t = _I64()
        self._check(self._L.aphgpu_server_submit(self._p, sim, _lib.ptr(v), dt,
                                                 ctypes.byref(t)), "submit")
        return t.value

    def wait(self, ticket, timeout_s=None):
        """Result of a step; with timeout_s, raises AphgpuError(TIMEOUT) if it
        has not completed by then (the ticket stays pending)."""
        r = StepResult()
        ms = -1.0 if timeout_s is None else 1e3 * timeout_s
        self._check(self._L.aphgpu_server_wait_timeout(self._p, ticket, ms, ctypes.byref(r)),
                    "wait")
        return r

    def state(self, sim):
        N = self.sizes[sim]
        a = np.empty(N)
        p = np.empty(N)
        self._check(self._L.aphgpu_server_get_state(self._p, sim, _lib.ptr(a), _lib.ptr(p)),
                    "get_state")
        return a, p

    def stats(self):
        st = Stats()
        self._check(self._L.aphgpu_server_get_stats(self._p, ctypes.byref(st)), "stats")
        return st
