// mlp_fused.cu - the control variate's network (64 -> 256 -> 256 -> 256 -> 256,
// GELU on the hidden layers, BF16 operands, FP32 accumulation) evaluated over
// many sites in one persistent launch on the tensor cores, with every
// activation kept on chip.
//
// The layer-by-layer path (mlp.cu: one k_tc_gemm per layer) writes each
// 128 x 256 BF16 activation tile to HBM and reads it back, and serialises the
// load, MMA and epilogue of every tile. Here one CTA per SM walks tiles of 128
// sites in pairs (two slots), so the tensor core works on one slot while the
// epilogue warps turn the other slot's accumulator into the next layer's
// operand:
//   warp 16 lane 0  TMA producer: the slot's feature tile [128][64] into the
//                   slot's activation buffer, then the weight panels of each
//                   layer (64 K-columns x 256 rows, 32 KB) through a 3-stage ring
//                   (the weights stay L2-resident: 416 KB for the network);
//   warp 17 lane 0  MMA issuer: per (slot, layer) tcgen05.mma M = 128, N = 256,
//                   K = 16 over the layer's K into the slot's 256-column TMEM
//                   accumulator (two slots: all 512 columns); tcgen05.commit
//                   frees weight stages, hands the accumulator to the epilogue
//                   and, after the last layer, frees the activation buffer;
//   warps 0..15     epilogue: warp w reads TMEM lanes 32 (w & 3) .. + 31 (one
//                   site each), columns 64 (w >> 2) .. + 63, in chunks of 32
//                   (tcgen05.ld.32x32b.x32). Hidden layers: + bias, GELU, BF16,
//                   stored into the slot's activation buffer in the K-major
//                   128-byte-swizzled layout the next MMA reads (the layout TMA
//                   writes). Last layer: + bias, then either the FP32 outputs
//                   to HBM or, for the site sum, a warp transpose-reduce of
//                   each 32 x 32 chunk (lane j ends with column j's sum over
//                   the warp's sites) added into per-lane partials (FP32 over
//                   8 tile pairs, then FP64).
// Order of work: (slot 0, layer 0), (slot 1, layer 0), (slot 0, layer 1), ...
// for each pair of tiles; the MMA and the epilogue both walk it, so the MMA
// of (slot s, layer l) waits only for the epilogue of (s, l - 1).
// Shared memory: 2 x 64 KB activation buffers + 3 x 32 KB weight stages.
// Every mbarrier wait gives up after two seconds, records a timeout in the
// status word and lets the block drain its copies and MMAs, free its TMEM and
// exit. The reference has no learned component: this evaluates the estimator's
// control variate only.
#include <cudaTypedefs.h>

#include <algorithm>

#include "tc_gemm.cuh"

using namespace leo2d;

namespace {

constexpr int kRows = 128;     // sites per tile (M of every MMA)
constexpr int kWidth = 256;    // layer width (N of every MMA)
constexpr int kKB = 64;        // K columns per weight stage / activation K block (one 128-byte swizzle span)
constexpr int kWStages = 3;
constexpr uint32_t kAKBlock = kRows * kKB * 2;             // 16 KB: one K block of an activation tile
constexpr uint32_t kABytes = kAKBlock * (kWidth / kKB);     // 64 KB: a 128 x 256 BF16 activation tile
constexpr uint32_t kWBytes = kWidth * kKB * 2;              // 32 KB: one weight panel
// 16 epilogue warps (four per TMEM lane quarter, 64 columns each): with 8 the
// epilogue issued at 57 % with two warps per scheduler and bounded the launch
constexpr int kEpiWarps = 16, kProducerWarp = 16, kMmaWarp = 17, kThreads = 32 * (kEpiWarps + 2);
constexpr int kEpiCols = kWidth / (kEpiWarps / 4);  // columns of one epilogue warp
constexpr uint32_t kIdesc = umma::idesc_bf16(kRows, kWidth);
constexpr size_t kSmemBytes = 2 * (size_t)kABytes + kWStages * (size_t)kWBytes + 1024;

__host__ __device__ constexpr int layer_kblocks(int l) { return l == 0 ? 1 : kWidth / kKB; }

struct FusedArgs {
  CUtensorMap tx;        // features [n][64] BF16, boxes 64 x 128
  CUtensorMap tw[4];     // W_l [256][in_l] BF16, boxes 64 x 256
  const float* bias[4];  // FP32 [256] each
  int64_t n;             // sites
  int64_t tiles;         // ceil(n / 128)
  float* y;              // [n][256] FP32 outputs, or null
  double* part;          // y null: [grid][4][256] FP64 column sums of the block's sites
  int* status;
};

// 32 consecutive FP32 columns of this thread's TMEM lane (32x32b shape), with
// the wait in the same statement so no use of the registers can move above it.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);  // lo at the lower address
  return *reinterpret_cast<const uint32_t*>(&p);
}

// (a, b) += (x, y) with one add.rn.f32x2 (the roundings of two FADDs)
__device__ __forceinline__ void add2(float& a, float& b, float x, float y) {
  unsigned long long r;
  asm("{\n\t.reg .b64 u, w;\n\tmov.b64 u, {%1, %2};\n\tmov.b64 w, {%3, %4};\n\t"
      "add.rn.f32x2 %0, u, w;\n\t}"
      : "=l"(r)
      : "f"(a), "f"(b), "f"(x), "f"(y));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// v[0..31] of every lane -> lane j returns sum over the warp's lanes of v[j]
// (five halving exchange steps, 31 shuffles).
__device__ __forceinline__ float warp_transpose_sum(float* v, int lane) {
#pragma unroll
  for (int w = 16; w >= 1; w >>= 1) {
    const bool up = (lane & w) != 0;
#pragma unroll
    for (int i = 0; i < w; ++i) {
      const float send = up ? v[i] : v[i + w];
      const float keep = up ? v[i + w] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, w);
    }
  }
  return v[0];
}

__global__ void __launch_bounds__(kThreads, 1) k_mlp_fused(const __grid_constant__ FusedArgs a) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* abuf = smem;                 // slot s at + s * kABytes
  unsigned char* wring = smem + 2 * kABytes;  // stage i at + i * kWBytes
  __shared__ __align__(8) uint64_t w_full[kWStages], w_empty[kWStages], x_full[2], x_empty[2], acc_full[2],
      epi_done[2], drain;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kWStages; ++i) {
      umma::bar_init(&w_full[i], 1);
      umma::bar_init(&w_empty[i], 1);
    }
    for (int s = 0; s < 2; ++s) {
      umma::bar_init(&x_full[s], 1);
      umma::bar_init(&x_empty[s], 1);
      umma::bar_init(&acc_full[s], 1);
      umma::bar_init(&epi_done[s], kEpiWarps);
    }
    umma::bar_init(&drain, 1);
    umma::bar_fence_init();
    abort_flag = 0;
  }
  if (warp == kMmaWarp) umma::tmem_alloc(&tmem_base, 2 * kWidth);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;

  const int64_t bid = blockIdx.x, grid = gridDim.x;
  const int64_t my_tiles = a.tiles > bid ? (a.tiles - bid + grid - 1) / grid : 0;
  const int iters = (int)((my_tiles + 1) / 2);
  // tile of slot s in pair iteration it (>= tiles: a padding tile, computed on
  // a real tile's data and discarded)
  auto tile_of = [&](int it, int s) { return bid + grid * (2 * (int64_t)it + s); };
  auto give_up = [&]() {
    abort_flag = 1;
    atomicExch(a.status, kStatusTimeout);
  };

  if (warp == kProducerWarp) {
    if (lane == 0) {
      uint32_t wi = 0;      // weight panels issued
      int x_issued[2] = {0, 0};
      bool ok = true;
      for (int it = 0; it < iters && ok; ++it)
        for (int l = 0; l < 4 && ok; ++l)
          for (int s = 0; s < 2 && ok; ++s) {
            if (abort_flag) {
              ok = false;
              break;
            }
            if (l == 0) {
              if (!umma::bar_wait(&x_empty[s], (uint32_t)(it & 1) ^ 1u)) {
                ok = false;
                break;
              }
              const int64_t t = std::min(tile_of(it, s), a.tiles - 1);
              umma::bar_expect_tx(&x_full[s], kAKBlock);
              umma::tma_load_2d(abuf + s * kABytes, &a.tx, 0, (int)(t * kRows), &x_full[s]);
              x_issued[s] = it + 1;
            }
            for (int kb = 0; kb < layer_kblocks(l); ++kb, ++wi) {
              const uint32_t st = wi % kWStages, ph = (wi / kWStages) & 1u;
              if (!umma::bar_wait(&w_empty[st], ph ^ 1u)) {
                ok = false;
                break;
              }
              umma::bar_expect_tx(&w_full[st], kWBytes);
              umma::tma_load_2d(wring + st * kWBytes, &a.tw[l], kb * kKB, 0, &w_full[st]);
            }
          }
      if (!ok) give_up();
      // every copy issued has landed before the block exits (the last copy of
      // each stage and slot; earlier ones were seen complete by their consumer)
      for (uint32_t i = wi > kWStages ? wi - kWStages : 0; i < wi; ++i)
        if (!umma::bar_wait(&w_full[i % kWStages], (i / kWStages) & 1u)) give_up();
      for (int s = 0; s < 2; ++s)
        if (x_issued[s] > 0 && !umma::bar_wait(&x_full[s], (uint32_t)(x_issued[s] - 1) & 1u)) give_up();
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {
      uint32_t wi = 0;
      bool ok = true;
      for (int it = 0; it < iters && ok; ++it)
        for (int l = 0; l < 4 && ok; ++l)
          for (int s = 0; s < 2 && ok; ++s) {
            const uint32_t j = 4u * (uint32_t)it + (uint32_t)l;  // item number on slot s
            if (abort_flag || (j > 0 && !umma::bar_wait(&epi_done[s], (j - 1) & 1u)) ||
                (l == 0 && !umma::bar_wait(&x_full[s], (uint32_t)it & 1u))) {
              ok = false;
              break;
            }
            umma::fence_after_sync();
            const uint32_t d = tmem + (uint32_t)(s * kWidth);
            const uint32_t a0 = umma::saddr(abuf + s * kABytes);
            for (int kb = 0; kb < layer_kblocks(l); ++kb, ++wi) {
              const uint32_t st = wi % kWStages, ph = (wi / kWStages) & 1u;
              if (!umma::bar_wait(&w_full[st], ph)) {
                ok = false;
                break;
              }
              umma::fence_after_sync();
              const uint32_t b0 = umma::saddr(wring + st * kWBytes);
#pragma unroll
              for (int k = 0; k < kKB / 16; ++k)
                umma::mma_bf16(d, umma::desc_k128(a0 + kb * kAKBlock + 32 * k), umma::desc_k128(b0 + 32 * k),
                               kIdesc, (kb | k) != 0 ? 1u : 0u);
              umma::mma_commit(&w_empty[st]);
            }
            if (!ok) break;
            umma::mma_commit(&acc_full[s]);
            if (l == 3) umma::mma_commit(&x_empty[s]);
          }
      if (!ok) give_up();
      // no MMA in flight once the block frees its TMEM
      umma::mma_commit(&drain);
      if (!umma::bar_wait(&drain, 0u)) give_up();
    }
  } else {
    // epilogue: site r = 32 q + lane of the tile, columns kEpiCols h .. + kEpiCols - 1
    const int q = warp & 3, h = warp >> 2, r = q * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    // site sums: FP32 over 8 tile pairs, then FP64 (the FP64 pipe is narrow)
    double csum[kEpiCols / 32];
    float fsum[kEpiCols / 32];
#pragma unroll
    for (int ci = 0; ci < kEpiCols / 32; ++ci) {
      csum[ci] = 0.0;
      fsum[ci] = 0.f;
    }
    // byte offset of K column k (multiple of 8) of this site in an activation buffer
    auto a_off = [&](int k) -> uint32_t {
      return (uint32_t)(k >> 6) * kAKBlock + (uint32_t)(r >> 3) * 1024u + (uint32_t)(r & 7) * 128u +
             ((uint32_t)(((k & 63) >> 3) ^ (r & 7)) << 4);
    };
    for (int it = 0; it < iters; ++it) {
      bool ok = true;
      for (int l = 0; l < 4 && ok; ++l)
        for (int s = 0; s < 2; ++s) {
          const uint32_t j = 4u * (uint32_t)it + (uint32_t)l;
          if (abort_flag || !umma::bar_wait(&acc_full[s], j & 1u)) {
            ok = false;
            break;
          }
          umma::fence_after_sync();
          const int64_t t = tile_of(it, s);
          const int64_t site = t * kRows + r;
          const bool valid = t < a.tiles && site < a.n;
          const uint32_t tacc = tmem + (uint32_t)(s * kWidth) + lane_off;
          const float* bl = a.bias[l];
          const uint32_t ab = umma::saddr(abuf + s * kABytes);
#pragma unroll
          for (int ci = 0; ci < kEpiCols / 32; ++ci) {
            const int c0 = h * kEpiCols + ci * 32;
            float v[32];
            tmem_ld32(tacc + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 32; i += 4) {
              const float4 b = __ldg(reinterpret_cast<const float4*>(bl + c0 + i));
              add2(v[i], v[i + 1], b.x, b.y);
              add2(v[i + 2], v[i + 3], b.z, b.w);
            }
            if (l < 3) {
              uint32_t pk[16];
#pragma unroll
              for (int i = 0; i < 16; ++i) {
                mlp_gelu2(v[2 * i], v[2 * i + 1]);
                pk[i] = pack_bf16x2(v[2 * i], v[2 * i + 1]);
              }
#pragma unroll
              for (int i = 0; i < 4; ++i)
                st_shared_v4(ab + a_off(c0 + 8 * i), pk[4 * i], pk[4 * i + 1], pk[4 * i + 2], pk[4 * i + 3]);
            } else if (a.y) {
              if (valid) {
                float4* dst = reinterpret_cast<float4*>(a.y + site * kWidth + c0);
#pragma unroll
                for (int i = 0; i < 8; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
              }
            } else {
              if (!valid)
#pragma unroll
                for (int i = 0; i < 32; ++i) v[i] = 0.f;
              fsum[ci] += warp_transpose_sum(v, lane);
            }
          }
          umma::fence_before_sync();
          if (l < 3) umma::fence_proxy_async();  // the activations feed the next MMA (async proxy)
          __syncwarp();
          if (lane == 0) umma::bar_arrive(&epi_done[s]);
        }
      if (!ok) {
        give_up();
        break;
      }
      if ((it & 7) == 7) {
#pragma unroll
        for (int ci = 0; ci < kEpiCols / 32; ++ci) {
          csum[ci] += (double)fsum[ci];
          fsum[ci] = 0.f;
        }
      }
    }
    if (!a.y) {
#pragma unroll
      for (int ci = 0; ci < kEpiCols / 32; ++ci)
        a.part[((size_t)bid * 4 + q) * kWidth + h * kEpiCols + ci * 32 + lane] = csum[ci] + (double)fsum[ci];
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (warp == kMmaWarp) umma::tmem_dealloc(tmem, 2 * kWidth);
}

// sums[c] = sum over the partial rows of part[.][c], in a fixed order.
__global__ void __launch_bounds__(256) k_fused_site_sums(const double* __restrict__ part, int rows,
                                                         double* __restrict__ sums) {
  const int c = threadIdx.x;
  double s = 0.0;
  for (int i = 0; i < rows; ++i) s += part[(size_t)i * kWidth + c];
  sums[c] = s;
}

}  // namespace

namespace leo2d {

void mlp_forward_fused(leo2d_ctx* ctx, const CUtensorMap& tx, const CUtensorMap* tw, const float* const* bias,
                       int64_t n, float* Y, double* sums_dev) {
  LEO_REQUIRE(n >= 1 && n < (int64_t(1) << 31), "fused MLP forward: n must be 1 .. 2^31 - 1");
  LEO_REQUIRE(Y || sums_dev, "fused MLP forward: no output");
  LEO_REQUIRE(kSmemBytes <= ctx->smem_optin, "fused MLP forward: shared memory per block too small");
  LEO_CUDA(cudaFuncSetAttribute(k_mlp_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes));
  FusedArgs a{};
  a.tx = tx;
  for (int l = 0; l < 4; ++l) {
    a.tw[l] = tw[l];
    a.bias[l] = bias[l];
  }
  a.n = n;
  a.tiles = (n + kRows - 1) / kRows;
  a.y = Y;
  a.status = ctx->status.p;
  const int grid = (int)std::min<int64_t>(ctx->sm_count, (a.tiles + 1) / 2);
  DevBuf<double> part(Y ? 0 : (size_t)grid * 4 * kWidth);
  a.part = part.p;
  launch(ctx, "mlp_fused", [&] { k_mlp_fused<<<grid, kThreads, kSmemBytes, ctx->stream>>>(a); });
  if (!Y)
    launch(ctx, "mlp_fused_sums",
           [&] { k_fused_site_sums<<<1, kWidth, 0, ctx->stream>>>(part.p, grid * 4, sums_dev); });
  ctx_sync(ctx);  // the partials are freed on return
}

}  // namespace leo2d
