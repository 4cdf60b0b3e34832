"""aphros_gb300: GB300-native projection-step hot path of aphros.

The product is libaphgpu.so (C ABI in include/aphgpu.h): the pressure
Poisson solve, PLIC VOF advection and height-function curvature as
hand-written CUDA for sm_103a.  This package holds its sources (csrc/), the
build script, the ctypes binding (_lib), host-side mirrors of the
reference's plug-in interfaces (linear, vof) and the synthetic workload
generator (workload).
"""
from . import _lib  # noqa: F401
from ._lib import AphgpuError, Context, default_conf  # noqa: F401

__all__ = ["Context", "AphgpuError", "default_conf"]
