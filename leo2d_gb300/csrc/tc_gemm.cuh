// tc_gemm.cuh - the tensor-core GEMM of the learned control variate:
//   D[M][N] = A[M][K] * B[N][K]^T (+ fused epilogue),
// A and B BF16, K-major (row-major with K contiguous), FP32 accumulation in
// tensor memory. Every MLP product maps onto it:
//   forward      A = activations [rows][in],  B = W [out][in]
//   input grad   A = dZ [rows][out],          B = W^T [in][out]
//   weight grad  A = dZ^T [out][rows],        B = activations^T [in][rows]
// (the epilogues write the transposed copies the next product needs).
//
// Kernel: persistent, one 128 x BN output tile at a time per block of 128
// threads. Lane 0 of warp 0 streams 128x64 and BNx64 BF16 tiles with TMA
// (128-byte swizzle) into a 4-stage ring; lane 0 of warp 1 issues
// tcgen05.mma (M = 128, N = BN, K = 16) into a BN-column TMEM accumulator and
// frees each stage with tcgen05.commit; all four warps then read the
// accumulator with tcgen05.ld (warp w owns rows 32w..32w+31) and apply the
// epilogue. Every wait gives up after two seconds, records a status and lets
// the block free its TMEM and exit.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"
#include "umma.cuh"

namespace leo2d {

enum GemmEpi : int {
  kEpiF32 = 0,       // out_f32 = D
  kEpiBias = 1,      // out_f32 = D + bias; with colsum: per-block column sums, nothing stored
  kEpiBiasGelu = 2,  // z = D + bias -> zout (FP32), h = gelu(z) -> out_bf16 and out_bf16_t
  kEpiGeluBwd = 3    // g = D * gelu'(zin) -> out_f32, out_bf16 and out_bf16_t
};

struct GemmArgs {
  int M, N, K;
  float* out_f32;              // [M][N]
  __nv_bfloat16* out_bf16;     // [M][N]
  __nv_bfloat16* out_bf16_t;   // [N][ld_t]
  int64_t ld_t;
  const float* bias;           // [N]
  const float* zin;            // [M][N]
  float* zout;                 // [M][N]
  double* colsum;              // [gridDim.x][N] (kEpiBias only, optional)
  int* status;
  // kEpiF32 only: the K range is split over k_splits work items per output tile;
  // item s writes split_buf + s*M*N and a second pass adds them into out_f32
  int k_splits;
  float* split_buf;
};

constexpr int kGemmBM = 128, kGemmBK = 64, kGemmStages = 4;

inline size_t gemm_smem_bytes(int BN) {
  return (size_t)kGemmStages * (kGemmBM + BN) * kGemmBK * 2 + 1024;
}

// Encodes a TMA map for a row-major BF16 matrix [rows][cols] (cols contiguous)
// with boxes of 64 columns x box_rows rows and the 128-byte swizzle.
void make_tmap_bf16(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int box_rows);
// The same with a row stride of `ld` elements (ld >= cols, ld*2 a multiple of 16).
void make_tmap_bf16_ld(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows);
// Blocks a GEMM of this output shape launches (one per SM at most).
int tc_gemm_grid(leo2d_ctx* ctx, int M, int N);

// TMA map for a row-major FP32 matrix [rows][cols] (row stride `ld` elements),
// boxes of 32 columns (128 bytes) x box_rows rows, 128-byte swizzle.
void make_tmap_f32(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows);

// out[M][N] (FP64, row-major) += A[M][K] * B[N][K]^T with FP32 operands, on the
// tensor cores: three TF32 products per K step (hi*hi + hi*lo + lo*hi), FP32
// accumulation over 2048 products at a time, added into FP64 partial tiles that
// are summed in a fixed order. K must be a multiple of 4 (16-byte rows). `ldo`:
// the row stride of out (<= 0: N).
void tc_gemm_f32x3_acc(leo2d_ctx* ctx, const float* A, const float* B, int M, int N, int64_t K, double* out,
                       int64_t ldo = 0);

// Sets the kernels' shared-memory attributes on the context's device (once;
// call before capturing GEMM launches into a graph).
void tc_gemm_prepare(leo2d_ctx* ctx);

// Launches D = A B^T with the epilogue; A is [M][K] behind ta, B is [N][K] behind tb.
void tc_gemm(leo2d_ctx* ctx, GemmEpi epi, const CUtensorMap& ta, const CUtensorMap& tb, const GemmArgs& g,
             int grid_cap = 0);

// The activation of the control variate's network: GELU(z) = z Phi(z) =
// z (1 + erf(z / sqrt 2)) / 2, with erf taken in the form of Abramowitz &
// Stegun, Handbook of Mathematical Functions (1964), formula 7.1.27: for x >= 0
//   erf(x) ~ 1 - (1 + a1 x + a2 x^2 + a3 x^3 + a4 x^4)^-4,  |error| <= 5e-4,
// extended as an odd function. This form (not the exact erf) defines the
// network: training, inference and the CPU oracle all evaluate it, so they
// agree to FP32 rounding. It costs four multiply-adds, two squarings and one
// reciprocal (rcp.approx) per activation; the fused forward evaluates 3 x 256
// of them per site, on two lanes at once (mlp_gelu2, fma.rn.f32x2). Every
// product and sum is an explicitly rounded operation, so the packed form and
// this scalar form agree bit for bit.
namespace mlp_act {
constexpr float kA1 = 0.278393f, kA2 = 0.230389f, kA3 = 0.000972f, kA4 = 0.078108f;
constexpr float kRsqrt2 = 0.70710678118654752f;
}  // namespace mlp_act

__device__ __forceinline__ float mlp_rcp(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
// 1 + a1 x + a2 x^2 + a3 x^3 + a4 x^4 (A&S 7.1.27)
__device__ __forceinline__ float mlp_erf_q(float x) {
  using namespace mlp_act;
  float p = __fmaf_rn(kA4, x, kA3);
  p = __fmaf_rn(p, x, kA2);
  p = __fmaf_rn(p, x, kA1);
  return __fmaf_rn(p, x, 1.0f);
}
// the network's erf(x) for x >= 0
__device__ __forceinline__ float mlp_erf_pos(float x) {
  float p = mlp_erf_q(x);
  p = __fmul_rn(p, p);
  p = __fmul_rn(p, p);
  return __fsub_rn(1.0f, mlp_rcp(p));
}
__device__ __forceinline__ float mlp_gelu(float z) {
  const float e = copysignf(mlp_erf_pos(__fmul_rn(fabsf(z), mlp_act::kRsqrt2)), z);
  const float hz = __fmul_rn(0.5f, z);
  return __fmaf_rn(hz, e, hz);
}
// d GELU / dz of that function: Phi(z) + z Phi'(z), with
// d erf / dx = 4 q'(x) / q(x)^5 for the form above
__device__ __forceinline__ float mlp_gelu_grad(float z) {
  using namespace mlp_act;
  const float x = fabsf(z) * kRsqrt2;
  const float e = copysignf(mlp_erf_pos(x), z);
  const float q = mlp_erf_q(x);
  const float q2 = q * q;
  const float dq = ((4.0f * kA4 * x + 3.0f * kA3) * x + 2.0f * kA2) * x + kA1;
  const float derf = 4.0f * dq / (q2 * q2 * q);
  return 0.5f * (1.0f + e) + z * 0.5f * kRsqrt2 * derf;
}

// GELU of two values at once (fma.rn.f32x2 / mul.rn.f32x2: the same roundings
// as mlp_gelu on each lane).
__device__ __forceinline__ void mlp_gelu2(float& a, float& b) {
  using namespace mlp_act;
  auto pk = [](float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
  };
  auto mul2 = [](unsigned long long x, unsigned long long y) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(x), "l"(y));
    return r;
  };
  auto fma2 = [](unsigned long long x, unsigned long long y, unsigned long long c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(x), "l"(y), "l"(c));
    return r;
  };
  const unsigned long long x = mul2(pk(fabsf(a), fabsf(b)), pk(kRsqrt2, kRsqrt2));
  unsigned long long p = fma2(pk(kA4, kA4), x, pk(kA3, kA3));
  p = fma2(p, x, pk(kA2, kA2));
  p = fma2(p, x, pk(kA1, kA1));
  p = fma2(p, x, pk(1.0f, 1.0f));
  p = mul2(p, p);
  p = mul2(p, p);
  float p0, p1;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(p0), "=f"(p1) : "l"(p));
  const float e0 = copysignf(__fsub_rn(1.0f, mlp_rcp(p0)), a);
  const float e1 = copysignf(__fsub_rn(1.0f, mlp_rcp(p1)), b);
  const unsigned long long hz = mul2(pk(a, b), pk(0.5f, 0.5f));
  const unsigned long long g = fma2(hz, pk(e0, e1), hz);
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(g));
}

// Forward of the control variate's network (64 -> 256 -> 256 -> 256 -> 256,
// GELU on the hidden layers) over n rows in one persistent launch with every
// activation kept on chip (mlp_fused.cu). tx: TMA map of the BF16 features
// [n][64] (boxes of 64 columns x 128 rows, 128-byte swizzle); tw[l]: TMA maps of
// the BF16 weights W_l [256][in_l] (boxes of 64 x 256); bias[l]: FP32 [256].
// Writes Y (FP32 [n][256]) or, with Y null, sums_dev[256] = the FP64 column
// sums of the outputs over the n rows (overwritten). n < 2^31.
void mlp_forward_fused(leo2d_ctx* ctx, const CUtensorMap& tx, const CUtensorMap* tw, const float* const* bias,
                       int64_t n, float* Y, double* sums_dev);

}  // namespace leo2d
