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

}  // namespace leo2d
