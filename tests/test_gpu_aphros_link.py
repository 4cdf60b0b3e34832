"""The reference-side adapters inside aphros itself (GPU).

aphros's own code is compiled from the staged reference sources
(oracle/ref/Makefile) and linked with the adapters (tests/aphros/Makefile):

  * aphros's linear-solver test (src/test/linear/main.cpp) selects the
    `gpu_cg`, `gpu` and `gpu_mixed` modules through `linsolver_symm`, as it
    selects `conjugate` (main.cpp:97-100), on 8 blocks of one rank; the
    reference test's own check (src/test/linear/test: the error against the
    exact solution within twice the conjugate solver's) must hold, and at a
    tight tolerance every solver reaches the same discrete solution.  The
    test's system is negative definite (aphros assembles the Laplacian
    with a negative diagonal); the multigrid solvers store its negation;
  * GpuVof and GpuHeights stepped by aphros's block framework equal aphros's
    Vof and curvature::Heights (oracle/_ref/ref_harness vof) on the same
    inputs and blocks.

Skipped where the reference sources are not staged.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from aphros_gb300 import build, workload
from conftest import REFERENCE, ROOT

pytestmark = pytest.mark.gpu

REF_SRC = os.path.join(REFERENCE, "src")
LINK_DIR = os.path.join(ROOT, "tests", "aphros")
OUT = os.path.join(LINK_DIR, "_build")
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


@pytest.fixture(scope="module")
def binaries():
    if not os.path.isdir(os.path.join(REF_SRC, "linear")):
        pytest.skip("aphros sources not staged")
    build.build_cuda()
    assert build.build_reference(), "reference build failed"
    jobs = str(min(16, os.cpu_count() or 4))
    r = subprocess.run(["make", "-C", LINK_DIR, "-j" + jobs], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return os.path.join(OUT, "t.linear"), os.path.join(OUT, "vof_gpu")


def _linear(exe, solver, tol, tmp_path):
    env = dict(os.environ, OMP_NUM_THREADS=str(min(8, os.cpu_count() or 1)))
    r = subprocess.run([exe, "--solver", solver, "--tol", repr(tol), "--maxiter", "100000",
                        "--mesh", "32", "--block", "16", "--verbose",
                        "--extra", "set string backend local"],
                       capture_output=True, text=True, cwd=tmp_path, env=env, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    out = {}
    for key in ("max_diff_exact", "residual", "iter"):
        m = re.search(key + r"=([-+0-9.eE]+)", r.stdout)
        assert m, r.stdout[-2000:]
        out[key] = float(m.group(1))
    return out


def test_linear_test_selects_gpu_modules(binaries, tmp_path):
    exe = binaries[0]
    conj = _linear(exe, "conjugate", 1e-5, tmp_path)
    # the reference's own expectation for conjugate (ref/conjugate/outdiff)
    assert conj["max_diff_exact"] < 2 * 6.926950e-03 + 1e-12
    for solver in ("gpu_cg", "gpu", "gpu_mixed"):
        res = _linear(exe, solver, 1e-5, tmp_path)
        assert res["residual"] < 1e-5, solver
        # src/test/linear/test: get_diff(out) < get_diff(ref) * 2 + 1e-12
        assert res["max_diff_exact"] < conj["max_diff_exact"] * 2 + 1e-12, (solver, res)


def test_linear_test_tight_solutions_agree(binaries, tmp_path):
    exe = binaries[0]
    conj = _linear(exe, "conjugate", 1e-11, tmp_path)
    for solver in ("gpu_cg", "gpu", "gpu_mixed"):
        res = _linear(exe, solver, 1e-11, tmp_path)
        assert res["residual"] < 1e-11, solver
        # the conjugate solver's error against the exact solution is a few
        # 1e-13 here (round-off of the solution's values); each solver's
        # stays within the same few round-off units of it
        assert res["max_diff_exact"] <= 1e-11, (solver, res, conj)


def test_gpu_vof_and_heights_in_aphros_equal_aphros(binaries, tmp_path):
    exe = binaries[1]
    case = workload.config("c1", n=32)
    dt = case.cfl_dt(0.5)
    case.alpha.tofile(str(tmp_path / "a.bin"))
    case.flux.tofile(str(tmp_path / "f.bin"))
    env = dict(os.environ, OMP_NUM_THREADS="4")
    steps = "4"
    r = subprocess.run([HARNESS, "vof", "32", "16", repr(case.h), repr(dt), steps, "a.bin",
                        "f.bin", "ref"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe, "32", "16", repr(dt), steps, "a.bin", "f.bin", "gpu"],
                       cwd=tmp_path, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    u_ref = np.fromfile(str(tmp_path / "ref.u"))
    k_ref = np.fromfile(str(tmp_path / "ref.k"))
    u = np.fromfile(str(tmp_path / "gpu.u"))
    k = np.fromfile(str(tmp_path / "gpu.k"))
    assert np.max(np.abs(u - u_ref)) <= 1e-12
    assert np.array_equal(np.isnan(k), np.isnan(k_ref))
    m = ~np.isnan(k_ref)
    assert m.sum() > 500
    assert np.max(np.abs(k[m] - k_ref[m])) <= 1e-7


@pytest.mark.parametrize("est", ["particles", "hybrid"])
def test_gpu_particle_curvature_in_aphros_equals_aphros(binaries, tmp_path, est):
    """GpuCurvature with the particle-string and hybrid estimators, stepped
    by aphros's block framework after GpuVof, against aphros's own
    curvature::Particles / curvature::Hybrid on one block of the same
    field (the reference's own multi-block result moves by up to 1e-11
    with the block layout; the device computes on the whole domain)."""
    exe = binaries[1]
    case = workload.config("c1", n=32)
    dt = case.cfl_dt(0.5)
    case.alpha.tofile(str(tmp_path / "a.bin"))
    case.flux.tofile(str(tmp_path / "f.bin"))
    env = dict(os.environ, OMP_NUM_THREADS="4", REF_CURV=est, APHGPU_CURV=est)
    r = subprocess.run([HARNESS, "vof", "32", "32", repr(case.h), repr(dt), "3", "a.bin",
                        "f.bin", "ref"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe, "32", "16", repr(dt), "3", "a.bin", "f.bin", "gpu"],
                       cwd=tmp_path, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    k_ref = np.fromfile(str(tmp_path / "ref.k"))
    k = np.fromfile(str(tmp_path / "gpu.k"))
    assert np.array_equal(np.isnan(k), np.isnan(k_ref))
    m = ~np.isnan(k_ref)
    assert m.sum() > 500
    rel = np.abs(k[m] - k_ref[m]) / np.abs(k_ref[m])
    print("%s: %d cells, max rel %.2e" % (est, m.sum(), rel.max()))
    assert rel.max() <= 1e-6
