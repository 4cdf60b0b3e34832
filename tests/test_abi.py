"""The C-ABI library loads and exports every entry point of include/*.h
(CPU only: no compute calls)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(aphgpu_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    from aphros_gb300 import build
    return build.build_cuda()


def test_header_declares_entry_points():
    names = _declared()
    for required in ("aphgpu_create", "aphgpu_destroy", "aphgpu_solve",
                     "aphgpu_set_system_expr", "aphgpu_assemble_projection",
                     "aphgpu_vof_step", "aphgpu_curvature"):
        assert required in names


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_exports_are_c_symbols(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (aphgpu_\w+)", out))
    assert set(_declared()) <= exported


def test_built_for_sm103a(libpath):
    """The device code of the library targets sm_103a only."""
    from aphros_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in build.ARCH
    assert os.path.getsize(libpath) > 100000


def test_conf_defaults_without_gpu(libpath):
    from aphros_gb300 import _lib
    c = _lib.default_conf()
    assert c.solver == _lib.SOLVER_MGPCG
    assert c.mg_pre == 2 and c.mg_post == 2
    assert c.miniter == 1


def test_create_rejects_bad_arguments(libpath):
    """Argument validation happens before any CUDA call."""
    from aphros_gb300 import _lib
    L = _lib.lib()
    p = ctypes.c_void_p()
    assert L.aphgpu_create(ctypes.byref(p), 2, 8, 8, 0.1, 0) == _lib.ERR_ARG
    assert L.aphgpu_create(ctypes.byref(p), 8, 8, 8, -1.0, 0) == _lib.ERR_ARG
    assert L.aphgpu_solve(None, None, None, None, None) == _lib.ERR_ARG
