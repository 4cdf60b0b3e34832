"""Host-side mirror of aphros's VOF advection solver and height-function
curvature estimator, running on the GPU through libaphgpu.

`Vof` follows AdvectionSolver/Vof (src/solver/advection.h:58-100,
src/solver/vof.h:62-112): StartStep / MakeIteration / FinishStep / PostStep,
GetField / GetAlpha / GetNormal / GetMask / GetColor / GetPlic.  `Heights`
follows curvature::Heights::CalcCurvature (src/solver/curv.h:70-90).
Scheme is weymouth (the VofPar default, src/solver/vof.h:44); with
`recolor=True` each MakeIteration also recolours the field as the
reference's default union-find labelling does (vof.ipp:546-578).
"""
import numpy as np

from . import _lib


class Plic:
    """generic::Plic (src/solver/advection.h:35-54), one layer."""

    def __init__(self, vof):
        self._vof = vof

    @property
    def vfcu(self):
        return self._vof.GetField()

    @property
    def vfcn(self):
        return self._vof.GetNormal()


class Vof:
    """Vof<M> on one periodic domain.

    m: linear.Mesh; fcu: initial volume fraction (ncells); fev: face fluxes
    (3 face blocks, see include/aphgpu.h); dt: time step; clipth: VofPar
    clipping threshold (default 1e-10); recolor: connected-component
    colours after every iteration (GetColor)."""

    def __init__(self, m, fcu, fev, t=0.0, dt=0.0, clipth=1e-10, device=0,
                 ctx=None, recolor=False):
        self.m = m
        self.ctx = ctx if ctx is not None else _lib.Context(m.n, m.h, device)
        self.fev = None if fev is None else np.ascontiguousarray(fev, dtype=np.float64)
        self.t = t
        self.dt = dt
        self.clipth = clipth
        self._u0 = np.ascontiguousarray(fcu, dtype=np.float64)
        self._started = False
        self._cache = None
        self.recolor = recolor

    def SetTimeStep(self, dt):
        self.dt = dt

    def GetTime(self):
        return self.t

    def GetTimeStep(self):
        return self.dt

    def SetFlux(self, fev):
        """Replaces the face fluxes (the owner's fev_ field)."""
        self.fev = None if fev is None else np.ascontiguousarray(fev, dtype=np.float64)

    def StartStep(self):
        # vof.ipp:177-195: reconstruct at t=0
        if not self._started:
            self.ctx.vof_init(self._u0, self.clipth)
            self._started = True
        self._cache = None

    def MakeIteration(self):
        self.ctx.vof_step(self.fev, self.dt)
        if self.recolor:
            self.ctx.vof_recolor()
        self._cache = None

    def FinishStep(self):
        self.t += self.dt

    def PostStep(self):
        pass

    def _state(self):
        if self._cache is None:
            self._cache = self.ctx.vof_get()
        return self._cache

    def GetField(self):
        return self._state()[0]

    def GetNormal(self):
        return self._state()[1]

    def GetAlpha(self):
        return self._state()[2]

    def GetMask(self):
        return self._state()[3]

    def GetColor(self):
        """Vof::GetColor (vof.ipp:741-743): -1 where no colour."""
        return self.ctx.vof_colors()

    def GetPlic(self):
        return Plic(self)


class Heights:
    """curvature::Heights: CalcCurvature(fck, plic, m) fills fck in place
    (NaN outside the interface)."""

    def CalcCurvature(self, fck, plic, m=None):
        k = plic._vof.ctx.curvature()
        fck[...] = k.reshape(np.shape(fck))
        return fck
