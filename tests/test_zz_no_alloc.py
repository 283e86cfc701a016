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


def _noalloc(ctx, torch, csr, P, R, seed, first):
    rp, col, val = csr.download()
    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(rp).to(dev)
    d_col = torch.from_numpy(col).to(dev)
    d_val = torch.from_numpy(val.astype(np.float32)).to(dev)
    stream = torch.cuda.current_stream(dev)
    d_mu = torch.full((R, P), float("nan"), dtype=torch.float64, device=dev)
    st = ctx.lib.leo2d_kpm_dos_noalloc(
        ctypes.c_void_p(d_rp.data_ptr()), ctypes.c_void_p(d_col.data_ptr()), ctypes.c_void_p(d_val.data_ptr()),
        csr.n, P, R, seed, first, ctypes.c_void_p(d_mu.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    return d_mu.cpu().numpy(), (rp, col, val)


def test_noalloc_matches_the_oracle():
    """The same recursion against the FP64 oracle on the same Philox vectors."""
    torch = pytest.importorskip("torch")
    from oracle import oracle
    with L.Context(0) as ctx:
        g = L.make_geom(model=L.MODEL_SIMPLE, size=24, angles_deg=(0.0, 3.0), energy_rescale=1.0)
        csr = ctx.build_csr(ctx.prepare(g))
        lo, hi = csr.bounds()
        csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
        P, R = 128, 3
        mu, (rp, col, val) = _noalloc(ctx, torch, csr, P, R, 8, 2)
        re, im = oracle.phase_vectors(8, 2, R, csr.n)
        o = (oracle.kpm_trace(rp, col, val, re, P, literal=False) +
             oracle.kpm_trace(rp, col, val, im, P, literal=False))
        assert np.max(np.abs(mu - o)) / np.max(np.abs(o)) < FP32_RTOL


def test_noalloc_narrow_blocks_on_a_large_flake():
    """About 2e5 orbitals: two 32-column buffers no longer fit the scratch array,
    so the call runs 16-column blocks (8 vectors each); 11 vectors take two blocks.
    Two calls in a row against leo2d_kpm_dos."""
    torch = pytest.importorskip("torch")
    with L.Context(0) as ctx:
        g = L.make_geom(model=L.MODEL_SIMPLE, size=190, max_R=290.0, angles_deg=(0.0, 1.1), energy_rescale=1.0)
        csr = ctx.build_csr(ctx.prepare(g))
        assert 131_072 < csr.n < 262_144  # 16 columns fit twice, 32 do not
        lo, hi = csr.bounds()
        csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
        P = 64
        for seed, first, R in [(2, 0, 11), (9, 4, 9)]:
            mu, _ = _noalloc(ctx, torch, csr, P, R, seed, first)
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
    # row counts past the int32 column range
    assert lib.leo2d_kpm_dos_noalloc(p, p, p, 1 << 31, 32, 1, 0, 0, p, None) == 1
    assert lib.leo2d_kpm_dos_noalloc(p, p, p, 0, 32, 1, 0, 0, p, None) == 1
    assert lib.leo2d_kpm_dos_noalloc(p, p, p, 4, 32, 0, 0, 0, p, None) == 1
