"""The reference-side adapter of INTEGRATION.md (linear::SolverGpu and its
ModuleLinear registration) compiles against aphros's own headers.  Runs
where the aphros sources are present (this check reads them from the
read-only reference tree); skipped elsewhere."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = "/root/reference/src"
ADAPTER = os.path.join(ROOT, "aphros_gb300", "adapter", "linear_aphgpu.cpp")


def test_adapter_matches_integration_doc():
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        blocks = re.findall(r"```cpp\n(.*?)```", f.read(), re.S)
    with open(ADAPTER) as f:
        assert f.read() == blocks[0] + "\n" + blocks[1]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_SRC, "linear")) or
                    shutil.which("g++") is None, reason="aphros sources or g++ absent")
def test_adapter_compiles_against_reference_headers(tmp_path):
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I" + REF_SRC,
           "-I" + os.path.join(ROOT, "include"), "-D_USE_MPI_=0", "-D_USE_OPENMP_=0",
           ADAPTER]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-3000:]
