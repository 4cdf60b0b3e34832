"""GPU test of aphgpu_cg_solve_noalloc, the CG entry point that allocates
nothing (for callers that cannot call cudaMalloc: a plug-in inside an
application that reserves the GPU's memory for its own pool, a step loop
with a fixed time budget where cudaMalloc would synchronize the device).

It is called through the C ABI on device arrays owned by the caller (torch
tensors here) and must give the same solution as the regular entry point
(aphgpu_solve with the plain CG solver) within the CG parity tolerance,
on two calls in a row (the second reuses the library's fixed scratch array
left over from the first).  This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from aphros_gb300 import _lib
from conftest import golden

pytestmark = pytest.mark.gpu


def _noalloc():
    L = _lib.lib()
    f = L.aphgpu_cg_solve_noalloc
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(_lib.Info)]
    f.restype = ctypes.c_int
    return f


def rel_l2(a, b):
    a = a - a.mean()
    b = b - b.mean()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_cg_matches_regular_entry_point():
    torch = pytest.importorskip("torch")
    fx = np.load(golden("proj16.npz"))
    n, h, tol = int(fx["n"]), float(fx["h"]), float(fx["tol"])
    expr = fx["expr_ref"]
    # regular entry point
    ctx = _lib.Context(n, h)
    ctx.set_system_expr(expr)
    x_ref, info_ref = ctx.solve(_lib.default_conf(solver=_lib.SOLVER_CG, tol=tol,
                                                  maxiter=100000))
    assert info_ref.converged
    # no-alloc entry point on caller-owned device arrays
    solve = _noalloc()
    d_e = torch.from_numpy(expr.copy()).cuda()
    d_x = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        d_x.fill_(123.0)  # the output is overwritten, whatever it held
        info = _lib.Info()
        rc = solve(n, n, n, h ** 3, d_e.data_ptr(), None, d_x.data_ptr(), tol, 1,
                   100000, 0, None, ctypes.byref(info))
        assert rc == _lib.OK, "call %d returned %d" % (call, rc)
        torch.cuda.synchronize()
        x = d_x.cpu().numpy()
        assert info.converged
        assert info.iter == info_ref.iter
        assert abs(info.residual - info_ref.residual) <= 1e-12 * info_ref.residual
        assert rel_l2(x, x_ref) <= 1e-12
        assert rel_l2(x, fx["p_ref"]) <= 1e-9
    # warm start from the solution (x0 aliases x): converges again, in a
    # small fraction of the cold-start iterations, and stays at the solution
    info = _lib.Info()
    rc = solve(n, n, n, h ** 3, d_e.data_ptr(), d_x.data_ptr(), d_x.data_ptr(), tol, 1,
               100000, 0, None, ctypes.byref(info))
    assert rc == _lib.OK and info.converged
    assert info.iter < info_ref.iter // 10
    torch.cuda.synchronize()
    assert rel_l2(d_x.cpu().numpy(), x_ref) <= 1e-9


def test_noalloc_rejects_oversized_grid():
    solve = _noalloc()
    info = _lib.Info()
    rc = solve(64, 64, 32, 1.0, 16, None, 16, 1e-6, 1, 10, 0, None, ctypes.byref(info))
    assert rc == _lib.ERR_ARG
