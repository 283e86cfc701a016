"""The tcgen05 tensor-core GEMM (D = A B^T, BF16 in, FP32 accumulate) against
a float64 product of the same BF16-rounded inputs.

Tolerance: FP32 accumulation over K terms of magnitude <= 1 in a different
order than the reference sum: 1e-5 of sqrt(K) plus relative 1e-5.
"""
import numpy as np
import pytest

import leo2d_gb300 as L

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """Round-to-nearest-even float32 -> BF16 bits (uint16)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 200, 136), (1000, 256, 512), (64, 64, 4096),
                                   (129, 257, 8), (2048, 512, 256)])
def test_tc_gemm(ctx, M, N, K):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    a = bf16_bits(rng.uniform(-1, 1, (M, K)))
    b = bf16_bits(rng.uniform(-1, 1, (N, K)))
    d = ctx.tc_gemm(a, b)
    ref = bf16_value(a) @ bf16_value(b).T
    np.testing.assert_allclose(d, ref, rtol=1e-5, atol=1e-5 * np.sqrt(K))


def test_tc_gemm_identity_structure(ctx):
    # exact small integers: every product and partial sum is exact in FP32
    M, N, K = 256, 256, 256
    rng = np.random.default_rng(1)
    a = rng.integers(-4, 5, (M, K)).astype(np.float32)
    b = rng.integers(-4, 5, (N, K)).astype(np.float32)
    d = ctx.tc_gemm(bf16_bits(a), bf16_bits(b))
    np.testing.assert_array_equal(d, (a.astype(np.float64) @ b.T.astype(np.float64)).astype(np.float32))


def test_tc_gemm_rejects_bad_k(ctx):
    with pytest.raises(L.Leo2dError, match="multiple of 8"):
        ctx.tc_gemm(np.zeros((4, 6), np.uint16), np.zeros((4, 6), np.uint16))


@pytest.mark.parametrize("N,K", [(8, 32), (32, 64), (32, 128), (64, 96), (128, 128), (256, 64)])
def test_tf32x3_product(ctx, N, K):
    """Three TF32 products per K step (A in tensor memory, B in swizzled shared
    memory): error within 2^-19 of sum_k |a||b| per element (three products
    keep about 22 bits; FP32 accumulation adds K * 2^-24)."""
    rng = np.random.default_rng(N + 7 * K)
    a = rng.normal(size=(128, K)).astype(np.float32)
    b = rng.normal(size=(N, K)).astype(np.float32)
    d = ctx.tc_gemm_tf32x3(a, b)
    ref = a.astype(np.float64) @ b.T.astype(np.float64)
    bound = np.abs(a).astype(np.float64) @ np.abs(b).T.astype(np.float64)
    assert np.all(np.abs(d - ref) <= 2.0 ** -19 * bound + 1e-30), np.max(np.abs(d - ref) / bound)
