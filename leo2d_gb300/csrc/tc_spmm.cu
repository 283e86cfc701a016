// tc_spmm.cu - tensor-core building blocks of the Chebyshev step: TF32 MMAs
// with the A operand in tensor memory (written from registers) and the B
// operand written into shared memory by the threads themselves (128-byte
// swizzled, K-major), three products per K step (hi*hi + hi*lo + lo*hi) so the
// result carries about 22 significant bits.
//
// leo2d_tc_gemm_tf32x3 exposes one 128-row product D = A B^T on host buffers.
#include "common.cuh"
#include "umma.cuh"

using namespace leo2d;

namespace {

// TF32 keeps the top 19 bits (sign, exponent, 10 mantissa bits).
__device__ __forceinline__ uint32_t tf32_hi(float x) { return __float_as_uint(x) & 0xFFFFE000u; }
__device__ __forceinline__ uint32_t tf32_lo(float x) {
  return __float_as_uint(x - __uint_as_float(__float_as_uint(x) & 0xFFFFE000u));
}

constexpr uint32_t kColD = 0, kColAhi = 256, kColAlo = 384;

// One block of 128 threads: D [128][N] = A [128][K] * B [N][K]^T, K <= 128
// (multiple of 32), N <= 256 (multiple of 8), N * K <= 24576.
__global__ void __launch_bounds__(128, 1) k_tf32x3(const float* __restrict__ A, const float* __restrict__ B, int N,
                                                   int K, float* __restrict__ D, int* status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* bhi = smem;
  unsigned char* blo = smem + (size_t)N * K * 4;
  __shared__ __align__(8) uint64_t done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    umma::bar_init(&done, 1);
    umma::bar_fence_init();
  }
  if (warp == 0) umma::tmem_alloc(&tmem_base, 512);
  // B (hi, lo) into the swizzled K-major layout
  for (int idx = threadIdx.x; idx < N * K; idx += 128) {
    const int n = idx / K, k = idx % K;
    const float x = B[idx];
    const uint32_t off = umma::k128_offset_b32(n, k, N);
    *reinterpret_cast<uint32_t*>(bhi + off) = tf32_hi(x);
    *reinterpret_cast<uint32_t*>(blo + off) = tf32_lo(x);
  }
  umma::fence_proxy_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  // A row of this thread (hi, lo) into tensor memory, 64 columns at a time
  const int m = threadIdx.x;
  for (int c0 = 0; c0 < K; c0 += 64) {
    uint32_t hi[64], lo[64];
#pragma unroll
    for (int j = 0; j < 64; ++j) {
      const float x = (c0 + j < K) ? A[(size_t)m * K + c0 + j] : 0.0f;
      hi[j] = tf32_hi(x);
      lo[j] = tf32_lo(x);
    }
    umma::tmem_st64(tmem + lane_base + kColAhi + c0, hi);
    umma::tmem_st64(tmem + lane_base + kColAlo + c0, lo);
  }
  umma::tmem_wait_st();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (threadIdx.x == 0) {
    const uint32_t idesc = umma::idesc_tf32(128, N);
    const uint32_t b0 = umma::saddr(bhi), b1 = umma::saddr(blo);
    for (int ks = 0; ks < K / 8; ++ks) {
      const uint32_t boff = (uint32_t)((ks >> 2) * N * 128 + (ks & 3) * 32);
      const uint32_t ahi = tmem + kColAhi + ks * 8, alo = tmem + kColAlo + ks * 8;
      umma::mma_tf32_ta(tmem + kColD, ahi, umma::desc_k128(b0 + boff), idesc, ks > 0 ? 1u : 0u);
      umma::mma_tf32_ta(tmem + kColD, ahi, umma::desc_k128(b1 + boff), idesc, 1u);
      umma::mma_tf32_ta(tmem + kColD, alo, umma::desc_k128(b0 + boff), idesc, 1u);
    }
    umma::mma_commit(&done);
  }
  __syncwarp();
  const bool ok = umma::bar_wait(&done, 0);
  umma::fence_after_sync();
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) atomicExch(status, kStatusTimeout);
  } else {
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      umma::tmem_ld16(tmem + lane_base + kColD + c0, v);
      for (int j = 0; j < 16 && c0 + j < N; ++j) D[(size_t)m * N + c0 + j] = v[j];
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

}  // namespace

extern "C" leo2d_status leo2d_tc_gemm_tf32x3(leo2d_ctx* ctx, const float* a, const float* b, int64_t N, int64_t K,
                                             float* d) {
  if (!ctx || !a || !b || !d) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_REQUIRE(K >= 32 && K <= 128 && K % 32 == 0, "K must be 32, 64, 96 or 128");
    LEO_REQUIRE(N >= 8 && N <= 256 && N % 8 == 0, "N must be a multiple of 8 in [8, 256]");
    LEO_REQUIRE(N * K <= 24576, "N * K must be <= 24576 (shared memory)");
    LEO_CUDA(cudaSetDevice(ctx->device));
    DevBuf<float> da((size_t)128 * K), db((size_t)N * K), dd((size_t)128 * N);
    h2d(ctx, da.p, a, (size_t)128 * K);
    h2d(ctx, db.p, b, (size_t)N * K);
    const size_t smem = (size_t)2 * N * K * 4 + 1024;
    LEO_CUDA(cudaFuncSetAttribute(k_tf32x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    launch(ctx, "tc_tf32x3", [&] {
      k_tf32x3<<<1, 128, smem, ctx->stream>>>(da.p, db.p, (int)N, (int)K, dd.p, ctx->status.p);
    });
    d2h(ctx, d, dd.p, (size_t)128 * N);
    ctx_check_status(ctx, "TF32x3 tensor-core product");
  });
}
