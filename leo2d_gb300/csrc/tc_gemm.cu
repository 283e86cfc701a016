// tc_gemm.cu - tcgen05 / TMA / TMEM GEMM with fused MLP epilogues (see tc_gemm.cuh).
#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>

#include "tc_gemm.cuh"

using namespace leo2d;

namespace {

constexpr int BM = kGemmBM, BK = kGemmBK, ST = kGemmStages, BN = 256;
constexpr uint32_t kABytes = BM * BK * 2, kBBytes = BN * BK * 2, kStage = kABytes + kBBytes;
constexpr uint32_t kIdesc = umma::idesc_bf16(BM, BN);

__device__ __forceinline__ float gelu(float z) { return mlp_gelu(z); }
__device__ __forceinline__ float gelu_grad(float z) { return mlp_gelu_grad(z); }

template <int EPI>
__global__ void __launch_bounds__(256, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, const GemmArgs g) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full[ST], empty[ST], done;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ double wsum[4][EPI == kEpiBias ? BN : 1];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      umma::bar_init(&full[s], 1);
      umma::bar_init(&empty[s], 1);
    }
    umma::bar_init(&done, 1);
    umma::bar_fence_init();
    abort_flag = 0;
  }
  if (EPI == kEpiBias)
    for (int i = threadIdx.x; i < 4 * BN; i += blockDim.x) (&wsum[0][0])[i] = 0.0;
  if (warp == 0) umma::tmem_alloc(&tmem_base, BN);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;

  const int m_tiles = (g.M + BM - 1) / BM, n_tiles = (g.N + BN - 1) / BN;
  const int nkb_all = (g.K + BK - 1) / BK;
  const int splits = g.k_splits > 1 ? g.k_splits : 1;
  const int kpb = (nkb_all + splits - 1) / splits;  // k-blocks per split
  uint32_t it = 0;
  int local = 0;
  for (int t = blockIdx.x; t < m_tiles * n_tiles * splits; t += gridDim.x, ++local) {
    const int split = t % splits, tile = t / splits;
    const int mt = tile % m_tiles, nt = tile / m_tiles;
    const int kb_first = split * kpb;
    const int nkb = max(0, min(nkb_all, kb_first + kpb) - kb_first);
    if (warp == 0 && lane == 0) {
      // producer: TMA tiles of A and B into the ring
      for (int kb = 0; kb < nkb && !abort_flag; ++kb) {
        const uint32_t i = it + kb, s = i % ST, ph = (i / ST) & 1u;
        if (!umma::bar_wait(&empty[s], ph ^ 1u)) {
          abort_flag = 1;
          break;
        }
        unsigned char* st = smem + (size_t)s * kStage;
        umma::bar_expect_tx(&full[s], kStage);
        umma::tma_load_2d(st, &ta, (kb_first + kb) * BK, mt * BM, &full[s]);
        umma::tma_load_2d(st + kABytes, &tb, (kb_first + kb) * BK, nt * BN, &full[s]);
      }
    } else if (warp == 1 && lane == 0) {
      // MMA issuer
      for (int kb = 0; kb < nkb && !abort_flag; ++kb) {
        const uint32_t i = it + kb, s = i % ST, ph = (i / ST) & 1u;
        if (!umma::bar_wait(&full[s], ph)) {
          abort_flag = 1;
          break;
        }
        umma::fence_after_sync();
        const uint32_t a0 = umma::saddr(smem + (size_t)s * kStage), b0 = a0 + kABytes;
#pragma unroll
        for (int k = 0; k < BK / 16; ++k)
          umma::mma_bf16(tmem, umma::desc_k128(a0 + 32 * k), umma::desc_k128(b0 + 32 * k), kIdesc,
                         (kb | k) != 0 ? 1u : 0u);
        umma::mma_commit(&empty[s]);
      }
      umma::mma_commit(&done);  // arrives when every MMA of this tile has finished
    }
    it += nkb;
    __syncwarp();
    const int late = umma::bar_wait(&done, (uint32_t)local & 1u) ? 0 : 1;
    if (__syncthreads_or(late | abort_flag)) {  // the whole block leaves together
      abort_flag = 1;
      break;
    }
    umma::fence_after_sync();

    // epilogue: thread = one row of the tile; warps w and w + 4 share the
    // tensor-memory lanes of quarter w and split the columns
    const int quarter = warp & 3, chalf = warp >> 2;
    const int r = mt * BM + quarter * 32 + lane;
    const bool row_ok = r < g.M;
    float* out32 = (EPI == kEpiF32 && splits > 1) ? g.split_buf + (size_t)split * g.M * g.N : g.out_f32;
    for (int c0 = chalf * (BN / 2); c0 < (chalf + 1) * (BN / 2); c0 += 16) {
      const int n0 = nt * BN + c0;
      if (n0 >= g.N) break;
      float v[16];
      if (nkb > 0) {
        umma::tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, v);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0.0f;  // an empty K range contributes nothing
      }
      const int cnt = min(16, g.N - n0);
      if (EPI == kEpiBias && g.colsum) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          double x = (row_ok && j < cnt) ? (double)(v[j] + g.bias[n0 + j]) : 0.0;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
          if (lane == 0 && j < cnt) wsum[quarter][c0 + j] += x;
        }
        continue;
      }
      if (!row_ok) continue;
      const size_t base = (size_t)r * g.N + n0;
      // full 16-column chunks of 16-byte-aligned rows go out as vectors
      const bool vec = cnt == 16 && (g.N & 15) == 0;
      if (EPI == kEpiF32 || EPI == kEpiBias) {
        float o[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) o[j] = EPI == kEpiBias && j < cnt ? v[j] + g.bias[n0 + j] : v[j];
        if (vec) {
#pragma unroll
          for (int j = 0; j < 16; j += 4)
            *reinterpret_cast<float4*>(out32 + base + j) = make_float4(o[j], o[j + 1], o[j + 2], o[j + 3]);
        } else {
          for (int j = 0; j < cnt; ++j) out32[base + j] = o[j];
        }
      } else if (EPI == kEpiBiasGelu) {
        float z[16];
        __nv_bfloat16 h[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          z[j] = j < cnt ? v[j] + g.bias[n0 + j] : 0.0f;
          h[j] = __float2bfloat16_rn(gelu(z[j]));
        }
        if (vec) {
          if (g.zout)
#pragma unroll
            for (int j = 0; j < 16; j += 4)
              *reinterpret_cast<float4*>(g.zout + base + j) = make_float4(z[j], z[j + 1], z[j + 2], z[j + 3]);
          if (g.out_bf16) {
            const uint4* hv = reinterpret_cast<const uint4*>(h);
            reinterpret_cast<uint4*>(g.out_bf16 + base)[0] = hv[0];
            reinterpret_cast<uint4*>(g.out_bf16 + base)[1] = hv[1];
          }
        } else {
          for (int j = 0; j < cnt; ++j) {
            if (g.zout) g.zout[base + j] = z[j];
            if (g.out_bf16) g.out_bf16[base + j] = h[j];
          }
        }
        if (g.out_bf16_t)
          for (int j = 0; j < cnt; ++j) g.out_bf16_t[(size_t)(n0 + j) * g.ld_t + r] = h[j];
      } else {  // kEpiGeluBwd
        float zi[16], gz[16];
        __nv_bfloat16 h[16];
        if (vec) {
#pragma unroll
          for (int j = 0; j < 16; j += 4) {
            const float4 q = *reinterpret_cast<const float4*>(g.zin + base + j);
            zi[j] = q.x; zi[j + 1] = q.y; zi[j + 2] = q.z; zi[j + 3] = q.w;
          }
        } else {
          for (int j = 0; j < 16; ++j) zi[j] = j < cnt ? g.zin[base + j] : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          gz[j] = v[j] * gelu_grad(zi[j]);
          h[j] = __float2bfloat16_rn(gz[j]);
        }
        if (vec) {
          if (g.out_f32)
#pragma unroll
            for (int j = 0; j < 16; j += 4)
              *reinterpret_cast<float4*>(g.out_f32 + base + j) = make_float4(gz[j], gz[j + 1], gz[j + 2], gz[j + 3]);
          if (g.out_bf16) {
            const uint4* hv = reinterpret_cast<const uint4*>(h);
            reinterpret_cast<uint4*>(g.out_bf16 + base)[0] = hv[0];
            reinterpret_cast<uint4*>(g.out_bf16 + base)[1] = hv[1];
          }
        } else {
          for (int j = 0; j < cnt; ++j) {
            if (g.out_f32) g.out_f32[base + j] = gz[j];
            if (g.out_bf16) g.out_bf16[base + j] = h[j];
          }
        }
        if (g.out_bf16_t)
          for (int j = 0; j < cnt; ++j) g.out_bf16_t[(size_t)(n0 + j) * g.ld_t + r] = h[j];
      }
    }
    umma::fence_before_sync();
    __syncthreads();
  }
  umma::fence_before_sync();
  __syncthreads();
  if (abort_flag && threadIdx.x == 0) atomicExch(g.status, kStatusTimeout);
  if (EPI == kEpiBias && g.colsum)
    for (int n = threadIdx.x; n < g.N && n < BN; n += blockDim.x)
      g.colsum[(size_t)blockIdx.x * g.N + n] = ((wsum[0][n] + wsum[1][n]) + wsum[2][n]) + wsum[3][n];
  if (warp == 0) umma::tmem_dealloc(tmem, BN);
}

// out[e] = sum over the K-range splits of part[s][e] (fixed order).
__global__ void k_split_sum(const float* __restrict__ part, int splits, int64_t total, float* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int k = 0; k < splits; ++k) s += part[(size_t)k * total + e];
    out[e] = s;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

}  // namespace

namespace leo2d {

void make_tmap_bf16(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int box_rows) {
  make_tmap_bf16_ld(map, base, rows, cols, cols, box_rows);
}

void make_tmap_bf16_ld(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
  auto fn = encode_fn();
  LEO_REQUIRE(fn != nullptr, "cuTensorMapEncodeTiled is not available from the driver");
  LEO_REQUIRE(((uintptr_t)base & 15) == 0, "tensor base must be 16-byte aligned");
  LEO_REQUIRE((ld * 2) % 16 == 0, "tensor row stride must be a multiple of 16 bytes");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)kGemmBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  LEO_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled rejected the tensor");
}

void tc_gemm_prepare(leo2d_ctx* ctx) {
  if (ctx->tc_gemm_ready) return;
  const int smem = (int)gemm_smem_bytes(BN);
  LEO_CUDA(cudaFuncSetAttribute(k_tc_gemm<kEpiF32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  LEO_CUDA(cudaFuncSetAttribute(k_tc_gemm<kEpiBias>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  LEO_CUDA(cudaFuncSetAttribute(k_tc_gemm<kEpiBiasGelu>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  LEO_CUDA(cudaFuncSetAttribute(k_tc_gemm<kEpiGeluBwd>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  ctx->tc_gemm_ready = true;
}

void tc_gemm(leo2d_ctx* ctx, GemmEpi epi, const CUtensorMap& ta, const CUtensorMap& tb, const GemmArgs& g,
             int grid_cap) {
  LEO_REQUIRE(g.M > 0 && g.N > 0 && g.K > 0, "empty GEMM");
  const size_t smem = gemm_smem_bytes(BN);
  const int splits = (epi == kEpiF32 && g.k_splits > 1 && g.split_buf) ? g.k_splits : 1;
  LEO_REQUIRE(splits == 1 || epi == kEpiF32, "only the plain product splits its K range");
  const int tiles = ((g.M + BM - 1) / BM) * ((g.N + BN - 1) / BN) * splits;
  int grid = std::min(tiles, ctx->sm_count);
  if (grid_cap > 0) grid = std::min(grid, grid_cap);
  tc_gemm_prepare(ctx);
  GemmArgs ga = g;
  ga.k_splits = splits;
  auto go = [&](auto kern) {
    launch(ctx, "tc_gemm", [&] { kern<<<grid, 256, smem, ctx->stream>>>(ta, tb, ga); });
  };
  switch (epi) {
    case kEpiF32:
      go(k_tc_gemm<kEpiF32>);
      if (splits > 1)
        launch(ctx, "tc_gemm_sum", [&] {
          k_split_sum<<<grid_for((int64_t)g.M * g.N, 256, (int64_t)ctx->sm_count * 8), 256, 0, ctx->stream>>>(
              g.split_buf, splits, (int64_t)g.M * g.N, g.out_f32);
        });
      return;
    case kEpiBias: return go(k_tc_gemm<kEpiBias>);
    case kEpiBiasGelu: return go(k_tc_gemm<kEpiBiasGelu>);
    case kEpiGeluBwd: return go(k_tc_gemm<kEpiGeluBwd>);
  }
  fail(LEO2D_ERR_BAD_ARG, "unknown GEMM epilogue");
}

int tc_gemm_grid(leo2d_ctx* ctx, int M, int N) {
  const int tiles = ((M + BM - 1) / BM) * ((N + BN - 1) / BN);
  return std::min(tiles, ctx->sm_count);
}

}  // namespace leo2d

// ---------------------------------------------------------------- C ABI

extern "C" leo2d_status leo2d_tc_gemm(leo2d_ctx* ctx, const uint16_t* a, const uint16_t* b, int64_t M, int64_t N,
                                      int64_t K, float* d) {
  if (!ctx || !a || !b || !d) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_REQUIRE(M >= 1 && N >= 1 && K >= 1 && M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31),
                "sizes must be in [1, 2^31)");
    LEO_REQUIRE(K % 8 == 0, "K must be a multiple of 8 (16-byte rows)");
    LEO_CUDA(cudaSetDevice(ctx->device));
    DevBuf<__nv_bfloat16> da((size_t)M * K), db((size_t)N * K);
    DevBuf<float> dd((size_t)M * N);
    h2d(ctx, reinterpret_cast<uint16_t*>(da.p), a, (size_t)M * K);
    h2d(ctx, reinterpret_cast<uint16_t*>(db.p), b, (size_t)N * K);
    CUtensorMap ta, tb;
    make_tmap_bf16(&ta, da.p, M, K, BM);
    make_tmap_bf16(&tb, db.p, N, K, BN);
    GemmArgs g{};
    g.M = (int)M;
    g.N = (int)N;
    g.K = (int)K;
    g.out_f32 = dd.p;
    g.status = ctx->status.p;
    tc_gemm(ctx, kEpiF32, ta, tb, g);
    d2h(ctx, d, dd.p, (size_t)M * N);
    ctx_check_status(ctx, "tensor-core GEMM");
  });
}

// ============================================================================
// FP32 GEMM from three TF32 products (the Kubo moment product mu = U B^T)
//
// Work items are (128 x 256 output tile, K range of at most kF3Chunk k-blocks of
// 32). Per item: warp 4 (one lane) streams 128x32 and 256x32 FP32 tiles with TMA
// into a 2-stage ring; warps 0-3 write each tile's low part x - tf32(x)
// elementwise into a parallel buffer (same swizzled layout); warp 5 (one lane)
// issues 4 K steps x 3 tcgen05.mma.kind::tf32 (A_hi B_hi + A_hi B_lo + A_lo B_hi;
// the tensor core reads the raw FP32 tile as its high part) into a 256-column TMEM
// accumulator; warps 0-3 then store the item's FP32 partial tile. A second kernel
// adds the partials of each output element in FP64 in a fixed order.
// ============================================================================

namespace {

constexpr int F3_BM = 128, F3_BN = 256, F3_BK = 32, F3_ST = 2, kF3Chunk = 4096, kF3Flush = 64;
constexpr uint32_t kF3A = F3_BM * F3_BK * 4, kF3B = F3_BN * F3_BK * 4;  // 16 KB, 32 KB
constexpr uint32_t kF3Raw = kF3A + kF3B, kF3Stage = 2 * kF3Raw;         // raw + low parts
constexpr uint32_t kF3Idesc = umma::idesc_tf32(F3_BM, F3_BN);

struct F3Args {
  int M, N;
  int64_t K;
  int m_tiles, n_tiles, splits;
  int64_t chunk_kb;  // k-blocks per work item
  double* partial;   // [items][128][256] FP64
  int* status;
};

__device__ __forceinline__ float tf32_low(float x) {
  return x - __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
}

// Work items: (output tile, K range of chunk_kb k-blocks). The FP32 accumulator
// is added into the item's FP64 tile every kF3Flush k-blocks (2048 products).
__global__ void __launch_bounds__(192, 1)
    k_tc_gemm_f32x3(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, const F3Args g) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full[F3_ST], conv[F3_ST], empty[F3_ST], tfull, tfree;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < F3_ST; ++s) {
      umma::bar_init(&full[s], 1);
      umma::bar_init(&conv[s], 128);
      umma::bar_init(&empty[s], 1);
    }
    umma::bar_init(&tfull, 1);
    umma::bar_init(&tfree, 128);
    umma::bar_fence_init();
    abort_flag = 0;
  }
  if (warp == 0) umma::tmem_alloc(&tmem_base, F3_BN);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const int64_t nkb = (g.K + F3_BK - 1) / F3_BK;
  const int64_t items = (int64_t)g.m_tiles * g.n_tiles * g.splits;
  uint32_t it = 0;   // k-blocks of this block so far (stage ring position)
  uint32_t sub = 0;  // accumulator sub-ranges of this block so far
  for (int64_t item = blockIdx.x; item < items && !abort_flag; item += gridDim.x) {
    const int split = (int)(item % g.splits);
    const int tile = (int)(item / g.splits);
    const int mt = tile % g.m_tiles, nt = tile / g.m_tiles;
    const int64_t kb0 = (int64_t)split * g.chunk_kb;
    const int nk = (int)(min(nkb, kb0 + g.chunk_kb) - kb0);
    const int nsub = (nk + kF3Flush - 1) / kF3Flush;
    if (warp == 4) {
      if (lane == 0)
        for (int k = 0; k < nk && !abort_flag; ++k) {
          const uint32_t i = it + k, s = i % F3_ST, ph = (i / F3_ST) & 1u;
          if (!umma::bar_wait(&empty[s], ph ^ 1u)) {
            abort_flag = 1;
            break;
          }
          unsigned char* st = smem + (size_t)s * kF3Stage;
          umma::bar_expect_tx(&full[s], kF3Raw);
          umma::tma_load_2d(st, &ta, (int)((kb0 + k) * F3_BK), mt * F3_BM, &full[s]);
          umma::tma_load_2d(st + kF3A, &tb, (int)((kb0 + k) * F3_BK), nt * F3_BN, &full[s]);
        }
    } else if (warp == 5) {
      if (lane == 0)
        for (int k = 0; k < nk && !abort_flag; ++k) {
          const uint32_t i = it + k, s = i % F3_ST, ph = (i / F3_ST) & 1u;
          const bool first_of_sub = (k % kF3Flush) == 0;
          const uint32_t q = sub + (uint32_t)(k / kF3Flush);  // this sub-range's index
          // the accumulator must have been read out by the previous sub-range's flush
          if (first_of_sub && q > 0 && !umma::bar_wait(&tfree, (q - 1) & 1u)) {
            abort_flag = 1;
            break;
          }
          if (!umma::bar_wait(&conv[s], ph)) {
            abort_flag = 1;
            break;
          }
          umma::fence_after_sync();
          const uint32_t a_hi = umma::saddr(smem + (size_t)s * kF3Stage), b_hi = a_hi + kF3A;
          const uint32_t a_lo = a_hi + kF3Raw, b_lo = b_hi + kF3Raw;
#pragma unroll
          for (int ks = 0; ks < F3_BK / 8; ++ks) {
            const uint32_t o = 32 * ks;
            umma::mma_tf32_ss(tmem, umma::desc_k128(a_hi + o), umma::desc_k128(b_hi + o), kF3Idesc,
                              (!first_of_sub || ks > 0) ? 1u : 0u);
            umma::mma_tf32_ss(tmem, umma::desc_k128(a_hi + o), umma::desc_k128(b_lo + o), kF3Idesc, 1u);
            umma::mma_tf32_ss(tmem, umma::desc_k128(a_lo + o), umma::desc_k128(b_hi + o), kF3Idesc, 1u);
          }
          umma::mma_commit(&empty[s]);
          if ((k % kF3Flush) == kF3Flush - 1 || k == nk - 1) umma::mma_commit(&tfull);
        }
    } else {
      // warps 0-3: low parts of each arriving stage; accumulator flushes into
      // this item's FP64 tile (one row per thread)
      double* acc = g.partial + (size_t)item * F3_BM * F3_BN + (size_t)threadIdx.x * F3_BN;
      for (int c = 0; c < F3_BN; c += 2) *reinterpret_cast<double2*>(acc + c) = make_double2(0.0, 0.0);
      for (int k = 0; k < nk; ++k) {
        const uint32_t i = it + k, s = i % F3_ST, ph = (i / F3_ST) & 1u;
        if (!umma::bar_wait(&full[s], ph)) {
          abort_flag = 1;
          break;
        }
        const float4* src = reinterpret_cast<const float4*>(smem + (size_t)s * kF3Stage);
        float4* dst = reinterpret_cast<float4*>(smem + (size_t)s * kF3Stage + kF3Raw);
        for (int e = threadIdx.x; e < (int)(kF3Raw / 16); e += 128) {
          const float4 x = src[e];
          dst[e] = make_float4(tf32_low(x.x), tf32_low(x.y), tf32_low(x.z), tf32_low(x.w));
        }
        umma::fence_proxy_async();
        umma::bar_arrive(&conv[s]);
        if ((k % kF3Flush) == kF3Flush - 1 || k == nk - 1) {
          const uint32_t q = sub + (uint32_t)(k / kF3Flush);
          if (!umma::bar_wait(&tfull, q & 1u)) {
            abort_flag = 1;
            break;
          }
          umma::fence_after_sync();
          for (int c0 = 0; c0 < F3_BN; c0 += 16) {
            float v[16];
            umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 16; j += 2) {
              double2 a = *reinterpret_cast<double2*>(acc + c0 + j);
              a.x += (double)v[j];
              a.y += (double)v[j + 1];
              *reinterpret_cast<double2*>(acc + c0 + j) = a;
            }
          }
          umma::fence_before_sync();
          umma::bar_arrive(&tfree);
        }
      }
    }
    it += nk;
    sub += nsub;
    __syncthreads();
  }
  // drain: the last sub-range's MMAs were waited for by its flush; a block that
  // gave up waits (bounded) for whatever it issued
  umma::fence_before_sync();
  __syncthreads();
  if (abort_flag && threadIdx.x == 0) atomicExch(g.status, kStatusTimeout);
  if (warp == 0) umma::tmem_dealloc(tmem, F3_BN);
}

// out[m][n] += sum over the K ranges of the FP64 partial tiles, fixed order.
__global__ void k_f3_reduce(const double* __restrict__ partial, int M, int N, int m_tiles, int splits,
                            double* __restrict__ out, int64_t ldo) {
  const int64_t total = (int64_t)M * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(e / N), n = (int)(e % N);
    const int tile = (n / F3_BN) * m_tiles + m / F3_BM;
    const size_t in_tile = (size_t)(m % F3_BM) * F3_BN + (n % F3_BN);
    double s = 0.0;
    for (int sp = 0; sp < splits; ++sp) s += partial[((size_t)tile * splits + sp) * F3_BM * F3_BN + in_tile];
    out[(int64_t)m * ldo + n] += s;
  }
}

}  // namespace

namespace leo2d {

void make_tmap_f32(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
  auto fn = encode_fn();
  LEO_REQUIRE(fn != nullptr, "cuTensorMapEncodeTiled is not available from the driver");
  LEO_REQUIRE(((uintptr_t)base & 15) == 0, "tensor base must be 16-byte aligned");
  LEO_REQUIRE((ld * 4) % 16 == 0, "tensor row stride must be a multiple of 16 bytes");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
  cuuint32_t box[2] = {(cuuint32_t)F3_BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  LEO_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled rejected the tensor");
}

void tc_gemm_f32x3_acc(leo2d_ctx* ctx, const float* A, const float* B, int M, int N, int64_t K, double* out,
                       int64_t ldo) {
  if (ldo <= 0) ldo = N;
  LEO_REQUIRE(M > 0 && N > 0 && K > 0, "empty GEMM");
  LEO_REQUIRE(K % 4 == 0, "K must be a multiple of 4");
  LEO_REQUIRE((K + F3_BK - 1) / F3_BK * F3_BK < (1ll << 31), "K too large for TMA coordinates");
  CUtensorMap ta, tb;
  make_tmap_f32(&ta, A, M, K, K, F3_BM);
  make_tmap_f32(&tb, B, N, K, K, F3_BN);
  F3Args g{};
  g.M = M;
  g.N = N;
  g.K = K;
  g.m_tiles = (M + F3_BM - 1) / F3_BM;
  g.n_tiles = (N + F3_BN - 1) / F3_BN;
  const int64_t nkb = (K + F3_BK - 1) / F3_BK;
  g.splits = (int)((nkb + kF3Chunk - 1) / kF3Chunk);
  g.chunk_kb = kF3Chunk;
  const int64_t items = (int64_t)g.m_tiles * g.n_tiles * g.splits;
  DevBuf<double> partial((size_t)items * F3_BM * F3_BN);
  g.partial = partial.p;
  g.status = ctx->status.p;
  const size_t smem = (size_t)F3_ST * kF3Stage + 1024;
  LEO_CUDA(cudaFuncSetAttribute(k_tc_gemm_f32x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = (unsigned)std::min<int64_t>(items, ctx->sm_count);
  launch(ctx, "cond_gemm", [&] { k_tc_gemm_f32x3<<<grid, 192, smem, ctx->stream>>>(ta, tb, g); });
  launch(ctx, "cond_gemm_sum", [&] {
    k_f3_reduce<<<grid_for((int64_t)M * N, 256, (int64_t)ctx->sm_count * 8), 256, 0, ctx->stream>>>(
        partial.p, M, N, g.m_tiles, g.splits, out, ldo);
  });
  ctx_check_status(ctx, "tensor-core FP32 product");
}

}  // namespace leo2d
