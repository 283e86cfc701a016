"""Error paths of the C ABI that a caller meets with bad input or too little
memory: each returns its status with a message and leaves the context usable.

- a CSR upload holding a NaN value: LEO2D_ERR_NONFINITE (the reference lets
  NaNs propagate silently);
- row counts past the int32 column range: LEO2D_ERR_BAD_ARG, checked before
  any array is read;
- a device allocation over the context's alloc_cap_mb: LEO2D_ERR_OOM.
"""
import ctypes

import numpy as np
import pytest

import leo2d_gb300 as L
from leo2d_gb300 import _abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def test_upload_rejects_nonfinite_values(ctx):
    rp = np.array([0, 2, 3], np.int64)
    col = np.array([0, 1, 1], np.int32)
    for bad in (np.nan, np.inf, -np.inf):
        val = np.array([1.0, bad, 2.0])
        with pytest.raises(L.Leo2dError) as e:
            ctx.upload_csr(rp, col, val)
        assert e.value.status == _abi.ERR_NONFINITE
        assert "non-finite" in str(e.value)
    csr = ctx.upload_csr(rp, col, np.array([1.0, 0.5, 2.0]))
    assert (csr.n, csr.nnz) == (2, 3)
    csr.close()


def test_upload_rejects_rows_past_int32(ctx):
    rp = np.zeros(4, np.int64)
    out = ctypes.c_void_p()
    for n in (1 << 31, (1 << 31) - 1, 0, -5):
        st = ctx.lib.leo2d_csr_upload(ctx.h, n, 0, rp.ctypes.data_as(ctypes.c_void_p), None, None, None, None,
                                      ctypes.byref(out))
        assert st == _abi.ERR_BAD_ARG
        assert not out.value
    assert b"n must be in" in ctx.lib.leo2d_last_error(ctx.h)


def test_alloc_cap_reports_oom(ctx):
    g = L.make_geom(model=L.MODEL_SIMPLE, size=30, angles_deg=(0.0, 2.0), energy_rescale=1.0)
    gp = ctx.prepare(g)
    ctx.set_option("alloc_cap_mb", 1)
    try:
        with pytest.raises(L.Leo2dError) as e:
            ctx.build_csr(gp)
        assert e.value.status == _abi.ERR_OOM
        assert "alloc_cap_mb" in str(e.value)
    finally:
        ctx.set_option("alloc_cap_mb", 0)
    csr = ctx.build_csr(gp)  # the same call without the cap
    assert csr.nnz * 8 > (1 << 20)
    lo, hi = csr.bounds()
    assert hi > lo
    csr.close()
