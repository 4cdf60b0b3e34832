"""Host-side mirror of aphros's linear-solver plug-in interface.

Same names, argument meaning and error behaviour as src/linear/linear.h:
`Solver.Solve(fc_system, fc_init, fc_sol) -> Info`, `Conf{tol, miniter,
maxiter}`, and the `ModuleLinear` registry that `linsolver_symm` selects from
(src/util/module.h:21-85, src/util/linear.ipp:22-26).  The registered names
are `gpu_cg` (plain CG, the algorithm of `conjugate`), `gpu` (MG-PCG, FP64)
and `gpu_mixed` (FP32 multigrid inside FP64 defect correction).  Every solve
runs on the GPU through libaphgpu's C ABI.
"""
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class Conf:
    """linear::Solver::Conf (src/linear/linear.h:21-25)."""
    tol: float = 0.0
    miniter: int = 1
    maxiter: int = 100


@dataclass
class Info:
    """linear::Solver::Info (src/linear/linear.h:27-30) plus GPU details."""
    residual: float
    iter: int
    inner_iter: int = 0
    converged: bool = False


class Mesh:
    """The part of MeshCartesian the solvers need: periodic cell counts and
    the (cubic) cell size."""

    def __init__(self, n, h):
        self.n = (n, n, n) if isinstance(n, int) else tuple(n)
        self.h = float(h)

    def GetCellSize(self):
        return (self.h, self.h, self.h)

    def ncells(self):
        return self.n[0] * self.n[1] * self.n[2]


_KINDS = {"gpu_cg": _lib.SOLVER_CG, "gpu": _lib.SOLVER_MGPCG,
          "gpu_mixed": _lib.SOLVER_MIXED}


class Solver:
    """linear::Solver (src/linear/linear.h:15-57)."""

    def __init__(self, conf):
        self.conf = conf

    def SetConf(self, conf):
        self.conf = conf

    def GetConf(self):
        return self.conf

    def Solve(self, fc_system, fc_init, fc_sol, m):
        raise NotImplementedError


# gpu_<prefix>_<name> variables that set context options (aphgpu_set_option)
_OPTIONS = {"cycle": _lib.OPT_CYCLE, "sweep_growth": _lib.OPT_SWEEP_GROWTH,
            "coarse_series": _lib.OPT_COARSE_SERIES}


class SolverGpu(Solver):
    """Drop-in `linsolver_symm gpu*`: the device state lives in a context
    keyed by the mesh size, like SolverConjugateCL::Shared
    (src/linear/conjugate_cl.ipp:155-187).

    fc_system: float64 array of 8 values per cell (FieldCell<Expr>),
    fc_init: initial guess or None (zero guess), may be fc_sol itself,
    fc_sol: output array, overwritten in place.
    Non-convergence is not an error (Info.iter > maxiter), as in CG; a
    non-symmetric system raises AphgpuError(ERR_NOT_SYMMETRIC).
    """

    def __init__(self, conf, kind="gpu", residual_max=False, device=0, options=None, **mg):
        super().__init__(conf)
        if kind not in _KINDS:
            raise ValueError("unknown solver kind '%s'" % kind)
        self.kind = kind
        self.residual_max = residual_max
        self.device = device
        self.mg = mg
        # context options by name: cycle, sweep_growth, coarse_series
        self.options = dict(options or {})
        self._ctx = None

    def context(self, m):
        if self._ctx is None or self._ctx.n != m.n or self._ctx.h != m.h:
            if self._ctx is not None:
                self._ctx.close()
            self._ctx = _lib.Context(m.n, m.h, self.device)
            for name, value in self.options.items():
                self._ctx.set_option(_OPTIONS[name], value)
        return self._ctx

    def native_conf(self):
        c = _lib.default_conf(solver=_KINDS[self.kind], tol=self.conf.tol,
                              miniter=self.conf.miniter, maxiter=self.conf.maxiter,
                              maxnorm=int(self.residual_max))
        for k, v in self.mg.items():
            setattr(c, k, v)
        return c

    def Solve(self, fc_system, fc_init, fc_sol, m):
        ctx = self.context(m)
        ctx.set_system_expr(fc_system)
        x0 = None if fc_init is None else np.array(fc_init, dtype=np.float64)
        x, info = ctx.solve(self.native_conf(), x0=x0)
        fc_sol[...] = x.reshape(fc_sol.shape)
        return Info(info.residual, info.iter, info.inner_iter, bool(info.converged))


class ModuleLinear:
    """Registry of linear solvers (src/linear/linear.h:59-76)."""

    _registry = {}

    def __init__(self, name):
        self.name = name

    @classmethod
    def Register(cls, module):
        cls._registry[module.name] = module

    @classmethod
    def GetInstance(cls, name):
        return cls._registry.get(name)

    @staticmethod
    def GetConf(var, prefix):
        """ModuleLinear::GetConf: hypre_<prefix>_{tol,maxiter,miniter}."""
        return Conf(tol=float(var["hypre_%s_tol" % prefix]),
                    maxiter=int(var["hypre_%s_maxiter" % prefix]),
                    miniter=int(var.get("hypre_%s_miniter" % prefix, 0)))

    def Make(self, var, prefix, m):
        raise NotImplementedError


class ModuleLinearGpu(ModuleLinear):
    def __init__(self, name):
        super().__init__(name)

    def Make(self, var, prefix, m):
        extra = {}
        for key in ("mg_pre", "mg_post", "mg_coarse_max", "inner_maxiter"):
            v = var.get("gpu_%s_%s" % (prefix, key))
            if v is not None:
                extra[key] = int(v)
        v = var.get("gpu_%s_inner_rtol" % prefix)
        if v is not None:
            extra["inner_rtol"] = float(v)
        options = {}
        for key in _OPTIONS:
            v = var.get("gpu_%s_%s" % (prefix, key))
            if v is not None:
                options[key] = int(v)
        return SolverGpu(self.GetConf(var, prefix), kind=self.name,
                         residual_max=bool(int(var.get("linsolver_%s_maxnorm" % prefix, 0))),
                         options=options, **extra)


for _name in _KINDS:
    ModuleLinear.Register(ModuleLinearGpu(_name))


def MakeLinearSolver(var, prefix, m):
    """ULinear::MakeLinearSolver (src/util/linear.ipp:7-28)."""
    name = var["linsolver_" + prefix]
    factory = ModuleLinear.GetInstance(name)
    if factory is None:
        raise RuntimeError("Solver not found: " + name)
    return factory.Make(var, prefix, m)
