"""The allocation-free trace entry point against leo2d_kpm_dos.

leo2d_kpm_dos_noalloc serves callers that may not allocate device memory
(stream-capture code, hosts whose device memory belongs to their own
allocator): it takes device pointers for the CSR and the moments and keeps its
scratch in a static device array. Its moments must equal those of
leo2d_kpm_dos for the same matrix, seed and vectors, within the FP32 tolerance
the other KPM tests use, on two calls in a row (the array keeps the previous
call's contents, which must not leak into the next result).
"""
import ctypes

import numpy as np
import pytest

import leo2d_gb300 as L

pytestmark = pytest.mark.gpu
FP32_RTOL = 1e-4


def test_noalloc_matches_kpm_dos_twice():
    torch = pytest.importorskip("torch")
    with L.Context(0) as ctx:
        g = L.make_geom(model=L.MODEL_SIMPLE, size=30, angles_deg=(0.0, 2.0), energy_rescale=1.0)
        csr = ctx.build_csr(ctx.prepare(g))
        lo, hi = csr.bounds()
        csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
        rp, col, val = csr.download()
        dev = torch.device("cuda:0")
        d_rp = torch.from_numpy(rp).to(dev)
        d_col = torch.from_numpy(col).to(dev)
        d_val = torch.from_numpy(val.astype(np.float32)).to(dev)
        P = 256
        stream = torch.cuda.current_stream(dev)
        for seed, first, R in [(21, 0, 6), (5, 3, 11)]:
            d_mu = torch.full((R, P), float("nan"), dtype=torch.float64, device=dev)
            st = ctx.lib.leo2d_kpm_dos_noalloc(
                ctypes.c_void_p(d_rp.data_ptr()), ctypes.c_void_p(d_col.data_ptr()),
                ctypes.c_void_p(d_val.data_ptr()), csr.n, P, R, seed, first,
                ctypes.c_void_p(d_mu.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
            assert st == 0
            torch.cuda.synchronize()
            mu = d_mu.cpu().numpy()
            ref = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP32, seed=seed,
                                        first_vector=first))
            assert np.isfinite(mu).all()
            assert np.max(np.abs(mu - ref)) / np.max(np.abs(ref)) < FP32_RTOL


def test_noalloc_rejects_oversize_and_bad_args():
    torch = pytest.importorskip("torch")
    lib = L._abi.load()
    dev = torch.device("cuda:0")
    d = torch.zeros(16, dtype=torch.int64, device=dev)
    p = ctypes.c_void_p(d.data_ptr())
    # 1e7 rows cannot fit the 32 MiB scratch array
    assert lib.leo2d_kpm_dos_noalloc(p, p, p, 10_000_000, 64, 1, 0, 0, p, None) == 1
    assert lib.leo2d_kpm_dos_noalloc(p, p, p, 4, 30, 1, 0, 0, p, None) == 1
    assert lib.leo2d_kpm_dos_noalloc(None, p, p, 4, 32, 1, 0, 0, p, None) == 1
