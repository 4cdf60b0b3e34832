"""The reference-side adapters (aphros_gb300/adapter/*.cpp: linear::SolverGpu
with its ModuleLinear registration, and the VOF and curvature classes)
compile against aphros's own headers.  Runs where the aphros sources are
staged (oracle/ref/stage_reference.sh); skipped elsewhere."""
import glob
import os
import shutil
import subprocess

import pytest

from conftest import REFERENCE, ROOT

REF_SRC = os.path.join(REFERENCE, "src")
ADAPTERS = sorted(glob.glob(os.path.join(ROOT, "aphros_gb300", "adapter", "*.cpp")))


def test_adapters_present():
    names = [os.path.basename(p) for p in ADAPTERS]
    assert "linear_aphgpu.cpp" in names


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_SRC, "linear")) or
                    shutil.which("g++") is None, reason="aphros sources or g++ absent")
@pytest.mark.parametrize("adapter", ADAPTERS, ids=os.path.basename)
def test_adapter_compiles_against_reference_headers(tmp_path, adapter):
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I" + REF_SRC,
           "-I" + os.path.join(ROOT, "include"), "-D_USE_MPI_=0", "-D_USE_OPENMP_=0",
           adapter]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-3000:]
