// tc_spmm.cu - tensor-core building blocks of the Chebyshev step: TF32 MMAs
// with the A operand in tensor memory (written from registers) and the B
// operand written into shared memory by the threads themselves (128-byte
// swizzled, K-major), three products per K step (hi*hi + hi*lo + lo*hi) so the
// result carries about 22 significant bits.
//
// leo2d_tc_gemm_tf32x3 exposes one 128-row product D = A B^T on host buffers.
#include "csr.cuh"
#include "kpm.cuh"
#include "step_kernels.cuh"
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

// ============================================================================
// The tensor-core Chebyshev step
//
// Format (built once per matrix from the locality-ordered copy, csr_build_tc):
// rows are grouped in tiles of 128; a tile's window is the sorted list of the
// distinct columns its rows touch (<= 1024, padded to a multiple of 64 with
// its last column); every row's entries are stored as (window position, FP32
// value) sorted by position, with the first entry of each 64-position chunk.
//
// Step (k_cheb_tc, one block of 256 threads per SM): for each tile and each
// 64-position chunk of its window, two stages in flight:
//   - the 64 window rows of T_n are read once (coalesced) and written as TF32
//     hi / lo parts into 128-byte-swizzled K-major shared memory (B operand);
//   - the two threads of each tile row scatter the row's chunk entries into a
//     scratch row, read it back and store its hi / lo parts into tensor memory
//     (A operand, lane = row);
//   - one thread issues 8 K steps x 3 TF32 MMAs (hi*hi, hi*lo, lo*hi) into a
//     C-column FP32 accumulator in tensor memory.
// The epilogue reads the accumulator (tcgen05.ld), forms T_{n+1} = a H T_n -
// T_{n-1}, writes it and accumulates <T_n|T_n>, <T_{n+1}|T_n> in FP64 per
// thread; block partials are reduced in fixed order by the next launch, as in
// the gather kernels. A row's entries gather nothing: T_n rows are reused from
// shared memory by every row of the tile.
// ============================================================================

namespace {

constexpr int kTcRows = 128, kTcMaxWin = 1024, kTcMaxEnt = 16384, kTcChunk = 64, kTcChunks = 16;
constexpr int kTcThreads = 256;

// Ascending bitonic sort of key[0, n) (n a power of two, >= 256) by a block of
// 256 threads, with an optional payload.
__device__ void bitonic_sort(uint32_t* key, uint32_t* val, int n) {
  for (int k = 2; k <= n; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool asc = (i & k) == 0;
          const uint32_t a = key[i], b = key[ixj];
          if ((a > b) == asc) {
            key[i] = b;
            key[ixj] = a;
            if (val) {
              const uint32_t t = val[i];
              val[i] = val[ixj];
              val[ixj] = t;
            }
          }
        }
      }
      __syncthreads();
    }
}

// Exclusive prefix sum of one int per thread over the block; *total gets the sum.
__device__ int block_excl_scan(int x, int* total) {
  __shared__ int s[kTcThreads];
  s[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < kTcThreads; o <<= 1) {
    const int v = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  const int incl = s[threadIdx.x];
  *total = s[kTcThreads - 1];
  __syncthreads();
  return incl - x;
}

__device__ __forceinline__ int lower_bound_u32(const uint32_t* a, int n, uint32_t x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// err[0]: bit 0 entries > 16384, bit 1 window > 1024, bit 2 row > 255 entries;
// err[1] most entries, err[2] widest window; wsum: sum of windows.
__global__ void __launch_bounds__(kTcThreads) k_tc_build(int64_t n, int64_t tiles, const int64_t* __restrict__ prow,
                                                         const int32_t* __restrict__ pcol,
                                                         const float* __restrict__ pval, int32_t* __restrict__ win,
                                                         int32_t* __restrict__ nwin, uint2* __restrict__ ent,
                                                         uint8_t* __restrict__ cstart, int* __restrict__ err,
                                                         unsigned long long* __restrict__ wsum) {
  extern __shared__ uint32_t tb_smem[];
  uint32_t* key = tb_smem;
  uint32_t* val = tb_smem + kTcMaxEnt;
  uint32_t* sw = tb_smem + 2 * kTcMaxEnt;
  __shared__ int64_t srp[kTcRows + 1];
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t r0 = t * kTcRows;
    const int rows = (int)min((int64_t)kTcRows, n - r0);
    for (int i = threadIdx.x; i <= rows; i += blockDim.x) srp[i] = prow[r0 + i];
    __syncthreads();
    const int64_t q0 = srp[0];
    const int E = (int)(srp[rows] - q0);
    if (E > kTcMaxEnt) {
      if (threadIdx.x == 0) atomicOr(&err[0], 1);
      __syncthreads();
      continue;
    }
    int P2 = 256;
    while (P2 < E) P2 <<= 1;
    for (int i = threadIdx.x; i < P2; i += blockDim.x) key[i] = i < E ? (uint32_t)pcol[q0 + i] : 0xFFFFFFFFu;
    __syncthreads();
    bitonic_sort(key, nullptr, P2);
    // distinct columns -> window
    const int per = P2 / kTcThreads;
    int cnt = 0;
    for (int j = 0; j < per; ++j) {
      const int i = threadIdx.x * per + j;
      const uint32_t k = key[i];
      if (k != 0xFFFFFFFFu && (i == 0 || key[i - 1] != k)) ++cnt;
    }
    int W = 0;
    int pos = block_excl_scan(cnt, &W);
    if (W > kTcMaxWin) {
      if (threadIdx.x == 0) atomicOr(&err[0], 2);
      __syncthreads();
      continue;
    }
    for (int j = 0; j < per; ++j) {
      const int i = threadIdx.x * per + j;
      const uint32_t k = key[i];
      if (k != 0xFFFFFFFFu && (i == 0 || key[i - 1] != k)) sw[pos++] = k;
    }
    __syncthreads();
    const int Wp = (W + kTcChunk - 1) / kTcChunk * kTcChunk;
    for (int w = threadIdx.x; w < Wp; w += blockDim.x) win[t * kTcMaxWin + w] = (int32_t)sw[w < W ? w : W - 1];
    if (threadIdx.x == 0) {
      nwin[t] = W;
      atomicMax(&err[1], E);
      atomicMax(&err[2], W);
      atomicAdd(wsum, (unsigned long long)W);
    }
    // entries sorted by (row, window position)
    for (int i = threadIdx.x; i < P2; i += blockDim.x) {
      if (i < E) {
        int lo = 0, hi = rows;  // row m with srp[m] <= q0 + i < srp[m + 1]
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (srp[mid] <= q0 + i) lo = mid;
          else hi = mid;
        }
        const int p = lower_bound_u32(sw, W, (uint32_t)pcol[q0 + i]);
        key[i] = ((uint32_t)lo << 16) | (uint32_t)p;
        val[i] = (uint32_t)i;
      } else {
        key[i] = 0xFFFFFFFFu;
        val[i] = 0;
      }
    }
    __syncthreads();
    bitonic_sort(key, val, P2);
    for (int i = threadIdx.x; i < E; i += blockDim.x)
      ent[q0 + i] = make_uint2(key[i] & 0xFFFFu, __float_as_uint(pval[q0 + val[i]]));
    for (int task = threadIdx.x; task < rows * kTcChunks; task += blockDim.x) {
      const int m = task / kTcChunks, c = task % kTcChunks;
      const int lb = lower_bound_u32(key, E, ((uint32_t)m << 16) | (uint32_t)(c * kTcChunk));
      const int rel = lb - (int)(srp[m] - q0);
      if (srp[m + 1] - srp[m] > 255) atomicOr(&err[0], 4);
      cstart[(r0 + m) * kTcChunks + c] = (uint8_t)min(rel, 255);
    }
    __syncthreads();
  }
}

struct TcArgs {
  int64_t n;
  const int64_t* rowptr;  // locality-ordered row pointers
  const uint2* ent;       // (window position, value bits)
  const uint8_t* cstart;  // [n][16]
  const int32_t* win;     // [tiles][1024]
  const int32_t* nwin;    // [tiles]
  const float* tn;        // T_n
  float* tp;              // T_{n-1} in (unless tprev), T_{n+1} out
  const float* tprev;
  int first;
  float alpha;            // 0: default (1 for the first step, else 2)
  int ent_cap;            // entries staged per tile (shared memory)
  double* partials;       // this step: [grid][2C]
  const double* prev_partials;
  double* prev_dots;
  int* status;
};

constexpr uint32_t kTcColD = 0, kTcColA = 128;  // A stage s: hi at 128 + 128 s, lo at +64

template <int C>
struct TcSmem {
  static constexpr uint32_t kB = kTcChunk * C * 4;              // one (hi or lo) B chunk
  static constexpr uint32_t kBAll = 4 * kB;                     // 2 stages x (hi, lo)
  static constexpr int kArowStride = 68;                        // floats per scratch row
  static constexpr uint32_t kArows = kTcRows * kArowStride * 4;
  static constexpr uint32_t kCst = kTcRows * kTcChunks;
  static constexpr uint32_t kWin = kTcMaxWin * 4;
  static constexpr uint32_t kRp = (kTcRows + 4) * 8;
  static constexpr uint32_t kFixed = kBAll + kArows + kCst + kWin + kRp;
};

template <int C>
__global__ void __launch_bounds__(kTcThreads, 1) k_cheb_tc(const TcArgs a) {
  static_assert(C == 32 || C == 64, "the tensor-core step takes 32 or 64 columns");
  using S = TcSmem<C>;
  constexpr int BV = kTcChunk * C / kTcThreads;  // window-row values per thread per chunk
  constexpr int CH = C / 2;                      // columns per thread in the epilogue
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* bbase = smem;  // [stage][hi, lo][kB]
  float* arows = reinterpret_cast<float*>(smem + S::kBAll);
  uint8_t* cst = smem + S::kBAll + S::kArows;
  int32_t* winl = reinterpret_cast<int32_t*>(smem + S::kBAll + S::kArows + S::kCst);
  int64_t* rp = reinterpret_cast<int64_t*>(smem + S::kBAll + S::kArows + S::kCst + S::kWin);
  uint2* ents = reinterpret_cast<uint2*>(smem + S::kFixed);
  __shared__ __align__(8) uint64_t load_bar, mma_bar[2], tile_bar, drain_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_nwin;
  __shared__ double red[2][4][2 * CH];

  if (a.prev_partials) reduce_prev<C, kTcThreads>(a.prev_partials, a.prev_dots, gridDim.x, blockIdx.x, gridDim.x);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m = tid & (kTcRows - 1), half = tid >> 7;
  if (tid == 0) {
    umma::bar_init(&load_bar, 1);
    umma::bar_init(&mma_bar[0], 1);
    umma::bar_init(&mma_bar[1], 1);
    umma::bar_init(&tile_bar, 1);
    umma::bar_init(&drain_bar, 1);
    umma::bar_fence_init();
  }
  if (warp == 0) umma::tmem_alloc(&tmem_base, 512);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  const float alpha = a.alpha != 0.0f ? a.alpha : (a.first ? 1.0f : 2.0f);
  const float* tprev = a.tprev ? a.tprev : a.tp;
  const int64_t tiles = (a.n + kTcRows - 1) / kTcRows;
  // dots: FP32 over kDotFlush tiles (one row each), then FP64 (the FP64 pipe is
  // a small fraction of the FP32 one)
  constexpr int kDotFlush = 16;
  double d0[CH], d1[CH];
  float e0[CH], e1[CH];
  int since_flush = 0;
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    d0[j] = d1[j] = 0.0;
    e0[j] = e1[j] = 0.f;
  }
  uint32_t chunk_ctr = 0;  // chunks issued by this block (stage = ctr & 1)
  uint32_t loads = 0;      // tile stagings issued (load_bar phases)
  int local = 0;           // tiles finished (tile_bar phases)
  bool failed = false;
  float xb[BV];            // the next chunk's window-row values (prefetched)

  // tile staging (one lane): row pointers, entries, chunk starts, window
  auto stage_tile = [&](int64_t t) {
    const int64_t r0 = t * kTcRows;
    const int rows = (int)min((int64_t)kTcRows, a.n - r0);
    const int W = a.nwin[t];
    s_nwin = W;
    const int Wp = (W + kTcChunk - 1) / kTcChunk * kTcChunk;
    const int64_t ra = r0 & ~1ll;
    const int64_t rcount = ((r0 + rows + 1 - ra) + 1) & ~1ll;
    const int64_t q0 = a.rowptr[r0], q1 = a.rowptr[r0 + rows];
    const int64_t qa = q0 & ~1ll;
    const int64_t qcount = ((q1 - qa) + 1) & ~1ll;
    const uint32_t cbytes = (uint32_t)((rows * kTcChunks + 15) & ~15);
    umma::bar_expect_tx(&load_bar, (uint32_t)(rcount * 8 + qcount * 8 + cbytes + Wp * 4));
    bulk_g2s(rp, a.rowptr + ra, (uint32_t)(rcount * 8), &load_bar);
    bulk_g2s(ents, a.ent + qa, (uint32_t)(qcount * 8), &load_bar);
    bulk_g2s(cst, a.cstart + r0 * kTcChunks, cbytes, &load_bar);
    bulk_g2s(winl, a.win + t * kTcMaxWin, (uint32_t)(Wp * 4), &load_bar);
  };
  // window rows of chunk k of the staged tile into registers
  auto load_b = [&](int k) {
#pragma unroll
    for (int j = 0; j < BV; ++j) {
      const int idx = tid + j * kTcThreads;
      const int w = idx / C, c = idx % C;
      xb[j] = __ldg(a.tn + (int64_t)winl[k * kTcChunk + w] * C + c);
    }
  };

  int64_t t = blockIdx.x;
  if (t < tiles) {
    if (tid == 0) stage_tile(t);
    ++loads;
    const int late = umma::bar_wait(&load_bar, 0u) ? 0 : 1;
    if (__syncthreads_or(late)) failed = true;
    else load_b(0);
  }
  for (; t < tiles && !failed; t += gridDim.x, ++local) {
    const int64_t r0 = t * kTcRows;
    const int rows = (int)min((int64_t)kTcRows, a.n - r0);
    const int W = s_nwin;
    const int nch = (W + kTcChunk - 1) / kTcChunk;
    const int64_t ra = r0 & ~1ll;
    const int64_t qa = rp[r0 - ra] & ~1ll;
    const bool row_ok = m < rows;
    const int rs = row_ok ? (int)(rp[r0 + m - ra] - qa) : 0;
    const int re = row_ok ? (int)(rp[r0 + m + 1 - ra] - qa) : 0;

    for (int k = 0; k < nch; ++k) {
      const uint32_t g = chunk_ctr++;
      const int s = (int)(g & 1u);
      // the stage's previous MMAs must be done before it is overwritten
      if (g >= 2) {
        const int late = umma::bar_wait(&mma_bar[s], ((g >> 1) - 1) & 1u) ? 0 : 1;
        if (__syncthreads_or(late)) {
          failed = true;
          break;
        }
      }
      unsigned char* bhi = bbase + (size_t)s * 2 * S::kB;
      unsigned char* blo = bhi + S::kB;
      // B: this chunk's window rows (prefetched) as hi / lo parts
#pragma unroll
      for (int j = 0; j < BV; ++j) {
        const int idx = tid + j * kTcThreads;
        const uint32_t off = umma::k128_offset_b32(idx % C, idx / C, C);
        *reinterpret_cast<uint32_t*>(bhi + off) = tf32_hi(xb[j]);
        *reinterpret_cast<uint32_t*>(blo + off) = tf32_lo(xb[j]);
      }
      if (k + 1 < nch) load_b(k + 1);  // in flight while this chunk is built
      // A: this thread's half (32 positions) of its row's chunk
      float* arow = arows + m * S::kArowStride + half * 32;
#pragma unroll
      for (int j = 0; j < 32; j += 4) *reinterpret_cast<float4*>(arow + j) = make_float4(0.f, 0.f, 0.f, 0.f);
      if (row_ok) {
        const int e0 = rs + cst[m * kTcChunks + k];
        const int e1 = k + 1 < kTcChunks ? rs + cst[m * kTcChunks + k + 1] : re;
        for (int e = e0; e < min(e1, re); ++e) {
          const uint2 en = ents[e];
          const int j = (int)en.x - k * kTcChunk - half * 32;
          if (j >= 0 && j < 32) arow[j] = __uint_as_float(en.y);
        }
      }
      uint32_t hi[32], lo[32];
#pragma unroll
      for (int j = 0; j < 32; j += 4) {
        const float4 v = *reinterpret_cast<const float4*>(arow + j);
        hi[j] = tf32_hi(v.x); lo[j] = tf32_lo(v.x);
        hi[j + 1] = tf32_hi(v.y); lo[j + 1] = tf32_lo(v.y);
        hi[j + 2] = tf32_hi(v.z); lo[j + 2] = tf32_lo(v.z);
        hi[j + 3] = tf32_hi(v.w); lo[j + 3] = tf32_lo(v.w);
      }
      const uint32_t acol = tmem + lane_base + kTcColA + 128u * s + 32u * half;
      umma::tmem_st32(acol, hi);
      umma::tmem_st32(acol + 64, lo);
      umma::tmem_wait_st();
      umma::fence_proxy_async();
      umma::fence_before_sync();
      __syncthreads();
      umma::fence_after_sync();
      if (tid == 0) {
        const uint32_t idesc = umma::idesc_tf32(kTcRows, C);
        const uint32_t b0 = umma::saddr(bhi), b1 = umma::saddr(blo);
        const uint32_t a_hi = tmem + kTcColA + 128u * s, a_lo = a_hi + 64;
#pragma unroll
        for (int ks = 0; ks < kTcChunk / 8; ++ks) {
          const uint32_t boff = (uint32_t)((ks >> 2) * C * 128 + (ks & 3) * 32);
          const uint32_t acc = (k > 0 || ks > 0) ? 1u : 0u;
          umma::mma_tf32_ta(tmem + kTcColD, a_hi + 8 * ks, umma::desc_k128(b0 + boff), idesc, acc);
          umma::mma_tf32_ta(tmem + kTcColD, a_hi + 8 * ks, umma::desc_k128(b1 + boff), idesc, 1u);
          umma::mma_tf32_ta(tmem + kTcColD, a_lo + 8 * ks, umma::desc_k128(b0 + boff), idesc, 1u);
        }
        umma::mma_commit(&mma_bar[s]);
        if (k + 1 == nch) umma::mma_commit(&tile_bar);  // the tile's accumulator
      }
    }
    if (failed) break;
    // the staging areas are free: stage the next tile while this one finishes
    const int64_t tn_next = t + gridDim.x;
    const bool has_next = tn_next < tiles;
    if (has_next && tid == 0) {
      umma::fence_proxy_async();  // the threads' reads of the staging areas precede the copies
      stage_tile(tn_next);
    }
    // epilogue operands of this tile's rows, loaded while the MMAs drain
    const int64_t off = (r0 + m) * C + half * CH;
    float4 xn[CH / 4], xp[CH / 4];
    if (row_ok) {
#pragma unroll
      for (int c0 = 0; c0 < CH; c0 += 4) {
        xn[c0 / 4] = __ldg(reinterpret_cast<const float4*>(a.tn + off + c0));
        xp[c0 / 4] = a.first ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4*>(tprev + off + c0);
      }
    }
    __syncwarp();
    const int late_t = umma::bar_wait(&tile_bar, (uint32_t)local & 1u) ? 0 : 1;
    int late_l = 0;
    if (has_next) late_l = umma::bar_wait(&load_bar, loads & 1u) ? 0 : 1;
    if (__syncthreads_or(late_t | late_l)) {
      failed = true;
      break;
    }
    if (has_next) {
      ++loads;
      load_b(0);  // the next tile's first window rows, in flight during this epilogue
    }
    umma::fence_after_sync();
    float v[CH];
#pragma unroll
    for (int c0 = 0; c0 < CH; c0 += 16) umma::tmem_ld16(tmem + lane_base + kTcColD + half * CH + c0, v + c0);
    if (row_ok) {
#pragma unroll
      for (int c0 = 0; c0 < CH; c0 += 4) {
        const float4 x = xn[c0 / 4], p = xp[c0 / 4];
        const float4 y = make_float4(alpha * v[c0] - p.x, alpha * v[c0 + 1] - p.y, alpha * v[c0 + 2] - p.z,
                                     alpha * v[c0 + 3] - p.w);
        *reinterpret_cast<float4*>(a.tp + off + c0) = y;
        e0[c0] += x.x * x.x; e1[c0] += y.x * x.x;
        e0[c0 + 1] += x.y * x.y; e1[c0 + 1] += y.y * x.y;
        e0[c0 + 2] += x.z * x.z; e1[c0 + 2] += y.z * x.z;
        e0[c0 + 3] += x.w * x.w; e1[c0 + 3] += y.w * x.w;
      }
    }
    if (++since_flush == kDotFlush) {  // block-uniform
      since_flush = 0;
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        d0[j] += (double)e0[j];
        d1[j] += (double)e1[j];
        e0[j] = e1[j] = 0.f;
      }
    }
    umma::fence_before_sync();
    __syncthreads();
  }
  // drain: every MMA and copy this block issued must finish before it exits
  if (tid == 0) {
    if (chunk_ctr > 0) {
      umma::mma_commit(&drain_bar);  // arrives once every earlier MMA of this thread is done
      umma::bar_wait(&drain_bar, 0u);
    }
    if (failed && loads > 0) umma::bar_wait(&load_bar, (loads - 1) & 1u);
  }
  if (tid == 0 && failed) atomicExch(a.status, kStatusTimeout);
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    d0[j] += (double)e0[j];
    d1[j] += (double)e1[j];
  }
  // block partials: rows (lanes) of each warp by shuffles, then the 4 warps of
  // each column half in order
#pragma unroll
  for (int j = 0; j < CH; ++j) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      d0[j] += __shfl_xor_sync(0xffffffffu, d0[j], o);
      d1[j] += __shfl_xor_sync(0xffffffffu, d1[j], o);
    }
  }
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      red[half][warp & 3][2 * j] = d0[j];
      red[half][warp & 3][2 * j + 1] = d1[j];
    }
  umma::fence_before_sync();
  __syncthreads();
  for (int tcol = tid; tcol < 2 * C; tcol += kTcThreads) {
    const int c = tcol >> 1, q = tcol & 1;
    const int h = c / CH, j = c % CH;
    const double s = ((red[h][0][2 * j + q] + red[h][1][2 * j + q]) + red[h][2][2 * j + q]) + red[h][3][2 * j + q];
    a.partials[(size_t)blockIdx.x * 2 * C + tcol] = s;
  }
  if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

}  // namespace

namespace leo2d {

void csr_drop_tc(leo2d_csr* csr) {
  csr->tc_built = false;
  csr->tc_tiles = 0;
  csr->tc_win.release();
  csr->tc_nwin.release();
  csr->tc_ent.release();
  csr->tc_cstart.release();
}

bool csr_build_tc(leo2d_ctx* ctx, leo2d_csr* csr) {
  LEO_REQUIRE(csr->reordered && csr->prow.p && csr->pcol.p && csr->pval32.p,
              "tensor-core tiles are built from the locality-ordered copy");
  csr_drop_tc(csr);
  const int64_t n = csr->n, nnz = csr->nnz;
  const int64_t tiles = (n + kTcRows - 1) / kTcRows;
  csr->tc_win.alloc((size_t)tiles * kTcMaxWin);
  csr->tc_nwin.alloc((size_t)tiles);
  csr->tc_ent.alloc((size_t)nnz + kCsrPad);
  LEO_CUDA(cudaMemsetAsync(csr->tc_ent.p + nnz, 0, kCsrPad * sizeof(uint2), ctx->stream));
  csr->tc_cstart.alloc((size_t)n * kTcChunks);
  DevBuf<int> err(3);
  DevBuf<unsigned long long> wsum(1);
  LEO_CUDA(cudaMemsetAsync(err.p, 0, 3 * sizeof(int), ctx->stream));
  LEO_CUDA(cudaMemsetAsync(wsum.p, 0, sizeof(unsigned long long), ctx->stream));
  const size_t smem = (size_t)(2 * kTcMaxEnt + kTcMaxWin) * 4;
  LEO_CUDA(cudaFuncSetAttribute(k_tc_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, (int64_t)ctx->sm_count);
  launch(ctx, "tc_build", [&] {
    k_tc_build<<<grid, kTcThreads, smem, ctx->stream>>>(n, tiles, csr->prow.p, csr->pcol.p, csr->pval32.p,
                                                        csr->tc_win.p, csr->tc_nwin.p, csr->tc_ent.p,
                                                        csr->tc_cstart.p, err.p, wsum.p);
  });
  int h[3] = {0, 0, 0};
  unsigned long long ws = 0;
  d2h(ctx, h, err.p, 3);
  d2h(ctx, &ws, wsum.p, 1);
  ctx_sync(ctx);
  if (h[0] != 0) {
    csr_drop_tc(csr);
    return false;
  }
  csr->tc_tiles = tiles;
  csr->tc_max_ent = h[1];
  csr->tc_max_win = h[2];
  csr->tc_mean_win = (double)ws / (double)tiles;
  csr->tc_patch = csr->reorder_patch;
  csr->tc_built = true;
  return true;
}

size_t tc_smem_bytes(const leo2d_csr* csr, int cols) {
  const uint32_t fixed = cols == 64 ? TcSmem<64>::kFixed : TcSmem<32>::kFixed;
  // at least 120 KB: one block per SM, so the block's 512 tensor-memory columns never wait on another block
  return std::max<size_t>(120 * 1024, 1024 + fixed + (size_t)(csr->tc_max_ent + 4) * 8);
}

void tc_launch_step(leo2d_ctx* ctx, const leo2d_csr* csr, int cols, unsigned grid, size_t smem, const float* tn,
                    float* tp, const float* tprev, int first, float alpha, double* partials,
                    const double* prev_partials, double* prev_dots) {
  TcArgs a{};
  a.n = csr->n;
  a.rowptr = csr->prow.p;
  a.ent = csr->tc_ent.p;
  a.cstart = csr->tc_cstart.p;
  a.win = csr->tc_win.p;
  a.nwin = csr->tc_nwin.p;
  a.tn = tn;
  a.tp = tp;
  a.tprev = tprev;
  a.first = first;
  a.alpha = alpha;
  a.ent_cap = csr->tc_max_ent + 4;
  a.partials = partials;
  a.prev_partials = prev_partials;
  a.prev_dots = prev_dots;
  a.status = ctx->status.p;
  auto go = [&](auto kern) {
    LEO_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    launch(ctx, "cheb_step", [&] { kern<<<grid, kTcThreads, smem, ctx->stream>>>(a); });
  };
  if (cols == 32) return go(k_cheb_tc<32>);
  if (cols == 64) return go(k_cheb_tc<64>);
  fail(LEO2D_ERR_BAD_ARG, "the tensor-core step takes 32 or 64 columns");
}

}  // namespace leo2d

extern "C" leo2d_status leo2d_csr_tc_info(const leo2d_csr* csr, int64_t* tiles, double* mean_window,
                                          int32_t* max_window, int32_t* max_tile_entries) {
  if (!csr) return LEO2D_ERR_BAD_ARG;
  if (tiles) *tiles = csr->tc_built ? csr->tc_tiles : 0;
  if (mean_window) *mean_window = csr->tc_built ? csr->tc_mean_win : 0.0;
  if (max_window) *max_window = csr->tc_built ? csr->tc_max_win : 0;
  if (max_tile_entries) *max_tile_entries = csr->tc_built ? csr->tc_max_ent : 0;
  return LEO2D_OK;
}
