"""Field dumps in aphros's raw + XMF format.

CPU: the XMF text of aphgpu_xmf_text equals dump::Xmf::WriteXmf's output for
the metadata dump::Raw::WriteWithXmf writes (golden texts from aphros's own
code, tests/golden/dumps.npz).  GPU: aphgpu_dump_raw writes the same raw
bytes as dump::Raw::WriteBlocks for each element type, and aphgpu_read_raw
reads them back."""
import os

import numpy as np
import pytest

from conftest import golden

CASES = [  # as tests/golden/make_golden.py XMF_CASES
    (16, 16, 16, 1 / 16, "vf", "vf.raw", "Double"),
    (32, 24, 16, 1 / 32, "p", "out/p_0001.raw", "Float"),
    (8, 8, 8, 0.125, "cl", "cl.raw", "UShort"),
    (48, 48, 48, 1 / 48, "kappa", "/tmp/k.raw", "Double"),
]


@pytest.fixture(scope="module")
def lib():
    from aphros_gb300 import _lib, build
    build.build_cuda()
    return _lib


@pytest.fixture(scope="module")
def fx():
    return np.load(golden("dumps.npz"))


def _dtype(lib, name):
    return {"Double": lib.DUMP_FLOAT64, "Float": lib.DUMP_FLOAT32, "UShort": lib.DUMP_UINT16}[name]


@pytest.mark.parametrize("q", range(len(CASES)))
def test_xmf_text_equals_reference(lib, fx, q):
    nx, ny, nz, h, name, binpath, typ = CASES[q]
    assert lib.xmf_text((nx, ny, nz), h, name, binpath, _dtype(lib, typ)) == str(fx["xmf%d" % q])


def test_xmf_text_rejects_bad_arguments(lib):
    with pytest.raises(lib.AphgpuError):
        lib.xmf_text((0, 4, 4), 0.25, "u", "u.raw")
    with pytest.raises(lib.AphgpuError):
        lib.xmf_text((4, 4, 4), 0.25, "u", "u.raw", dtype=7)


@pytest.mark.gpu
@pytest.mark.parametrize("typ", ["Double", "Float", "UShort"])
def test_dump_raw_bytes_and_read_back(lib, fx, tmp_path, typ):
    v = np.asarray(fx["values"], dtype=np.float64)
    ctx = lib.Context((3, 4, 5), 0.25)
    ctx.set_solution(v)
    raw = tmp_path / ("p_%s.raw" % typ)
    ctx.dump_raw(lib.FIELD_PRESSURE, raw, "p", _dtype(lib, typ))
    assert np.array_equal(np.fromfile(raw, dtype=np.uint8), fx["raw_" + typ])
    xmf = tmp_path / ("p_%s.xmf" % typ)
    assert xmf.read_text() == lib.xmf_text((3, 4, 5), 0.25, "p", str(raw), _dtype(lib, typ))
    ctx.set_solution(np.zeros(60))
    ctx.read_raw(lib.FIELD_PRESSURE, xmf)
    back = ctx.get_solution()
    want = {"Double": v, "Float": v.astype(np.float32).astype(np.float64),
            "UShort": np.trunc(v)}[typ]
    assert np.array_equal(back, want)
    ctx.close()


@pytest.mark.gpu
def test_volume_fraction_checkpoint(lib, tmp_path):
    """A served simulation's volume fraction survives a dump and a read
    bit for bit, and the next step from the restored field equals the step
    from the original (the restored context has made as many steps, so that
    both sweep in the same order)."""
    from aphros_gb300 import workload
    case = workload.config("c1", n=32)
    a = lib.Context(32, case.h)
    a.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    a.vof_init(case.alpha)
    dt = case.cfl_dt(0.5)
    a.vof_step(case.flux, dt)
    raw = tmp_path / "vf.raw"
    a.dump_raw(lib.FIELD_VF, raw, "vf")
    b = lib.Context(32, case.h)
    b.assemble_projection(case.alpha, case.rho1, case.rho2, case.flux, case.dt)
    b.vof_init(np.zeros(32 ** 3))
    b.vof_step(case.flux, dt)
    b.read_raw(lib.FIELD_VF, os.path.splitext(raw)[0] + ".xmf")
    ua = a.vof_get()[0]
    assert np.array_equal(b.vof_get()[0], ua)
    a.vof_step(case.flux, dt)
    b.vof_step(case.flux, dt)
    assert np.array_equal(a.vof_get()[0], b.vof_get()[0])
    # dimensions that differ from the context's, and a field not yet there
    c = lib.Context(16, 1 / 16)
    with pytest.raises(lib.AphgpuError):
        c.read_raw(lib.FIELD_VF, os.path.splitext(raw)[0] + ".xmf")
    c.vof_init(np.zeros(16 ** 3))
    with pytest.raises(lib.AphgpuError):
        c.read_raw(lib.FIELD_VF, os.path.splitext(raw)[0] + ".xmf")
    for ctx in (a, b, c):
        ctx.close()
