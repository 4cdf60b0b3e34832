import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# aphros as staged by oracle/ref/stage_reference.sh
REFERENCE = os.environ.get(
    "APHROS_REFERENCE", os.path.join(ROOT, "baseline", "_ref", "aphros"))


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (sm_103a) and libaphgpu.so")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the native libraries once per session if they are missing."""
    from aphros_gb300 import build
    build.build_gen()
    build.build_oracle()
    yield


def golden(name):
    return os.path.join(GOLDEN, name)


def read_table(name):
    """Rows of a golden text table: (inputs, outputs[, expectation])."""
    rows = []
    with open(golden(name)) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            rows.append([p.strip() for p in line.split("|")])
    return rows
