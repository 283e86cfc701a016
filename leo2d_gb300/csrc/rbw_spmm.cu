// rbw_spmm.cu - the row-block Chebyshev step with shared-memory windows
// (FP32, 32 columns).
//
// The row-block step (rb_spmm.cu) gathers each T_n row through L1 once per
// row block. Its gathers miss L1 about one time in four (each tile of blocks
// touches each of its distinct T_n rows once) and every miss is an L1
// request held by the load/store unit, so the step stalls on those misses
// long before the L1 data pipe or HBM saturate. This variant moves the misses
// to the bulk-copy path instead:
//
// Format (built once from the row blocks): blocks are taken in tiles of TB
// blocks; a tile's window is the sorted list of the distinct columns of its
// slots, and each slot stores its column's position in the window in place of
// the column itself.
//   rbw_roff  int64[tiles + 1]   first run of each tile
//   rbw_runs  int32[2 * runs]    (first column, rows) of each run of consecutive
//                                T_n rows of the window (gaps of one row are
//                                copied with the run)
//   rbw_wrows int32[tiles]       rows of each tile's window
//   rbw_data  as rb_data, with window positions in place of columns
// Kernel (one block per SM, TB compute warps + 1 producer warp)
//   The producer warp fills a 2..4-stage ring: for each tile, the block
//   offsets and the tile's slots (positions and values) with cp.async.bulk, and
//   the window - one cp.async.bulk per run of consecutive T_n rows (a few dozen
//   per tile: one copy per row would be bound by the copy issue rate) - all
//   completing on the stage's mbarrier. Compute
//   warp w takes block w of the tile and reads its T_n rows from the window in
//   shared memory (a quarter-warp reads one 128-byte row: one wavefront), with
//   the lane layout, accumulation, reduce-scatter and epilogue of the row-block
//   step. Compute warps release a stage on an "empty" mbarrier; the producer
//   waits for it before refilling. Every wait is bounded (two seconds or the
//   context's poll limit) and reports a status; copies in flight land before
//   the block exits.
#include <algorithm>
#include <cmath>

#include "kpm.cuh"

using namespace leo2d;

#include "step_kernels.cuh"

namespace {

#include "rb_common.cuh"

constexpr int kRbwTile = 16;          // row blocks per tile (= compute warps)
constexpr int kRbwBuildThreads = 256;
constexpr int kRbwMaxSlots = 8192;    // slots of one tile (build limit)
constexpr int kRbwMaxWin = 2048;      // window rows of one tile (build limit)
constexpr int kRbwMaxRuns = 1024;     // runs of one tile's window (build limit)
constexpr int kRbwGap = 1;            // gaps of up to this many rows are copied with the runs

// ---------------------------------------------------------------- format build

__device__ void bitonic_sort_u32(uint32_t* key, int n) {
  for (int k = 2; k <= n; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool up = (i & k) == 0;
          const uint32_t x = key[i], y = key[ixj];
          if ((x > y) == up) {
            key[i] = y;
            key[ixj] = x;
          }
        }
      }
      __syncthreads();
    }
}

__device__ int rbw_block_scan(int x, int* total) {
  __shared__ int s[kRbwBuildThreads];
  s[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < kRbwBuildThreads; o <<= 1) {
    const int v = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  const int incl = s[threadIdx.x];
  *total = s[kRbwBuildThreads - 1];
  __syncthreads();
  return incl - x;
}

// The window of a tile is copied as runs of consecutive T_n rows; gaps of up
// to kRbwGap rows between distinct columns are copied too, so that runs are
// long (with the patch ordering a tile's columns fall in a few dozen runs).
// Pass 0: nrun[t] = runs of tile t, and wrows[t] = rows copied (distinct
// columns plus gap rows). Pass 1: writes the runs (first column, length) at
// runs + 2 roff[t] and, in rbw_data (a copy of rb_data), each slot's window
// position over its column.
// err[0]: bit 0 a tile with more than kRbwMaxSlots slots, bit 1 more than
// kRbwMaxWin rows copied or kRbwMaxRuns runs; err[1] most rows copied;
// wsum: rows copied over all tiles.
__global__ void __launch_bounds__(kRbwBuildThreads) k_rbw_build(int64_t nrb, int tb, const int64_t* __restrict__ off,
                                                                const unsigned char* __restrict__ rb_data, int pass,
                                                                int64_t* __restrict__ nrun,
                                                                int32_t* __restrict__ wrows,
                                                                const int64_t* __restrict__ roff,
                                                                int32_t* __restrict__ runs,
                                                                unsigned char* __restrict__ rbw_data,
                                                                int* __restrict__ err,
                                                                unsigned long long* __restrict__ wsum) {
  extern __shared__ uint32_t wk[];  // kRbwMaxSlots sorted columns, the distinct ones, their window positions
  uint32_t* win = wk + kRbwMaxSlots;
  int* posx = reinterpret_cast<int*>(win + kRbwMaxWin);
  int* rstart = posx + kRbwMaxWin;  // first column of each run
  __shared__ int64_t soff[kRbwTile + 1];
  const int64_t tiles = (nrb + tb - 1) / tb;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t b0 = t * tb;
    const int nb = (int)min((int64_t)tb, nrb - b0);
    if (threadIdx.x <= kRbwTile) soff[threadIdx.x] = off[b0 + min((int)threadIdx.x, nb)];
    __syncthreads();
    const int K = (int)(soff[nb] - soff[0]);
    if (K > kRbwMaxSlots) {
      if (threadIdx.x == 0) {
        atomicOr(&err[0], 1);
        if (pass == 0) nrun[t] = 0;
      }
      __syncthreads();
      continue;
    }
    int P2 = kRbwBuildThreads;
    while (P2 < K) P2 <<= 1;
    // the columns of the tile's slots (block by block)
    for (int i = threadIdx.x; i < P2; i += blockDim.x) {
      uint32_t c = 0xFFFFFFFFu;
      if (i < K) {
        int b = 0;
        while (b + 1 < nb && soff[b + 1] - soff[0] <= i) ++b;
        const int64_t s = soff[0] + i;
        c = (uint32_t)reinterpret_cast<const int32_t*>(rb_data + soff[b] * kRbSlotBytes)[s - soff[b]];
      }
      wk[i] = c;
    }
    __syncthreads();
    bitonic_sort_u32(wk, P2);
    // distinct columns, compacted into win[0, W)
    const int per = P2 / kRbwBuildThreads;
    const int i0 = threadIdx.x * per;
    int cnt = 0;
    for (int j = 0; j < per; ++j) {
      const int i = i0 + j;
      if (i < K && (i == 0 || wk[i] != wk[i - 1])) ++cnt;
    }
    int W = 0;
    int pos = rbw_block_scan(cnt, &W);
    if (W > kRbwMaxWin) {
      if (threadIdx.x == 0) {
        atomicOr(&err[0], 2);
        if (pass == 0) nrun[t] = 0;
      }
      __syncthreads();
      continue;
    }
    for (int j = 0; j < per; ++j) {
      const int i = i0 + j;
      if (i < K && (i == 0 || wk[i] != wk[i - 1])) win[pos++] = wk[i];
    }
    __syncthreads();
    // runs and window positions: element j starts a run when the gap to the
    // previous column exceeds kRbwGap rows; smaller gaps are copied
    const int wper = (W + kRbwBuildThreads - 1) / kRbwBuildThreads;
    const int j0 = threadIdx.x * wper;
    int starts = 0, rows = 0;
    for (int j = j0; j < min(W, j0 + wper); ++j) {
      const uint32_t d = j == 0 ? 0u : win[j] - win[j - 1];
      if (j == 0 || d > (uint32_t)kRbwGap + 1) {
        ++starts;
        rows += 1;
      } else {
        rows += (int)d;
      }
    }
    int R = 0, Wx = 0;
    int run_at = rbw_block_scan(starts, &R);
    int row_at = rbw_block_scan(rows, &Wx);
    if (pass == 0) {
      if (threadIdx.x == 0) {
        if (Wx > kRbwMaxWin || R > kRbwMaxRuns) atomicOr(&err[0], 2);
        nrun[t] = R;
        wrows[t] = Wx;
        atomicMax(&err[1], Wx);
        atomicAdd(wsum, (unsigned long long)Wx);
      }
      __syncthreads();
      continue;
    }
    // run starts and positions, then (once every start is known) the runs
    int ra = run_at, rw = row_at;
    for (int j = j0; j < min(W, j0 + wper); ++j) {
      const uint32_t d = j == 0 ? 0u : win[j] - win[j - 1];
      if (j == 0 || d > (uint32_t)kRbwGap + 1) {
        rstart[ra++] = (int)win[j];
        rw += 1;
      } else {
        rw += (int)d;
      }
      posx[j] = rw - 1;
    }
    __syncthreads();
    int32_t* rout = runs + 2 * roff[t];
    ra = run_at;
    for (int j = j0; j < min(W, j0 + wper); ++j) {
      const uint32_t d = j == 0 ? 0u : win[j] - win[j - 1];
      if (j == 0 || d > (uint32_t)kRbwGap + 1) ++ra;
      const bool last = j == W - 1 || win[j + 1] - win[j] > (uint32_t)kRbwGap + 1;
      if (last) {
        rout[2 * (ra - 1)] = rstart[ra - 1];
        rout[2 * (ra - 1) + 1] = (int32_t)(win[j] - (uint32_t)rstart[ra - 1] + 1);
      }
    }
    __syncthreads();
    // window position of every slot, over its column
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
      int b = 0;
      while (b + 1 < nb && soff[b + 1] - soff[0] <= i) ++b;
      const int64_t s = soff[0] + i;
      const uint32_t c = (uint32_t)reinterpret_cast<const int32_t*>(rb_data + soff[b] * kRbSlotBytes)[s - soff[b]];
      int lo = 0, hi = W;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (win[mid] < c) lo = mid + 1;
        else hi = mid;
      }
      reinterpret_cast<int32_t*>(rbw_data + soff[b] * kRbSlotBytes)[s - soff[b]] = posx[lo];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- the step

struct RbwArgs {
  int64_t n;
  int64_t nrb;
  const int64_t* __restrict__ off;
  const unsigned char* __restrict__ data;
  const int64_t* __restrict__ roff;  // first run of each tile
  const int32_t* __restrict__ runs;  // (first column, rows) per run
  const int32_t* __restrict__ wrows; // rows copied per tile
  const float* __restrict__ tn;
  float* __restrict__ tp;
  const float* __restrict__ tprev;
  int first;
  float alpha;
  double* __restrict__ partials;
  const double* __restrict__ prev_partials;
  double* __restrict__ prev_dots;
  int stages;
  int chunk;
  int off_bytes;    // offsets region of a stage
  int data_bytes;   // slots region of a stage
  int stage_bytes;  // offsets + slots + window rows, multiple of 128
  uint64_t spin_limit;
  int* status;
  int never_wait;
};

template <int TB, bool PACKED, int U>
__global__ void __launch_bounds__((TB + 1) * 32, 1) k_cheb_rbw(const __grid_constant__ RbwArgs a) {
  constexpr int C = 32;
  constexpr int NT = (TB + 1) * 32;
  constexpr int kMaxStages = 4;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kMaxStages];
  __shared__ __align__(8) uint64_t empty[kMaxStages];
  __shared__ int issued[kMaxStages];
  __shared__ __align__(8) uint64_t never;
  const int bid = (int)blockIdx.x, nblk = (int)gridDim.x;
  if (a.prev_partials) reduce_prev<C, NT>(a.prev_partials, a.prev_dots, nblk, bid, nblk);

  const int nst = a.stages;
  const int64_t n_tiles = (a.nrb + TB - 1) / TB;
  if (threadIdx.x == 0) {
    for (int i = 0; i < nst; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], TB);
      issued[i] = 0;
    }
    mbar_init(&never, 1);
    mbar_fence_init();
  }
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t chunk = a.chunk;
  auto tile_of = [&](int64_t i) -> int64_t {
    return ((int64_t)bid + (i / chunk) * (int64_t)nblk) * chunk + i % chunk;
  };

  double d0 = 0.0, d1 = 0.0;  // column `lane` (compute warps)

  if (warp == TB) {
    // ---- producer
    for (int it = 0;; ++it) {
      const int64_t tile = tile_of(it);
      if (tile >= n_tiles) break;
      const int stage = it % nst;
      bool ok = true;
      if (it >= nst) ok = bounded_wait(&empty[stage], (uint32_t)((it / nst) - 1) & 1u, a.spin_limit);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) atomicExch(a.status, leo2d::kStatusTimeout);
        break;
      }
      const int64_t b0 = tile * TB, b1 = min(a.nrb, b0 + TB);
      const int64_t ba = b0 & ~1ll;
      const int64_t ocount = ((b1 + 1 - ba) + 1) & ~1ll;
      const int64_t s0 = a.off[b0], s1 = a.off[b1];
      const int64_t r0 = a.roff[tile];
      const int R = (int)(a.roff[tile + 1] - r0);
      const int Wx = a.wrows[tile];
      const uint32_t dbytes = (uint32_t)((s1 - s0) * kRbSlotBytes);
      unsigned char* st = smem + (size_t)stage * a.stage_bytes;
      unsigned char* win = st + a.off_bytes + a.data_bytes;
      if (lane == 0) {
        issued[stage] += 1;
        mbar_expect_tx(&full[stage], (uint32_t)(ocount * 8) + dbytes + (uint32_t)Wx * 128u);
        bulk_g2s(st, a.off + ba, (uint32_t)(ocount * 8), &full[stage]);
        if (dbytes) bulk_g2s(st + a.off_bytes, a.data + s0 * kRbSlotBytes, dbytes, &full[stage]);
      }
      __syncwarp();
      // one copy per run, at the run's window position (a warp prefix sum of lengths)
      int base = 0;
      for (int k0 = 0; k0 < R; k0 += 32) {
        const int k = k0 + lane;
        int start = 0, len = 0;
        if (k < R) {
          start = __ldg(a.runs + 2 * (r0 + k));
          len = __ldg(a.runs + 2 * (r0 + k) + 1);
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        if (len > 0)
          bulk_g2s(win + (size_t)(base + incl - len) * 128, a.tn + (size_t)(uint32_t)start * C, (uint32_t)len * 128u,
                   &full[stage]);
        base += __shfl_sync(0xffffffffu, incl, 31);
      }
    }
  } else {
    // ---- compute warps
    const int g = lane >> 3, q = lane & 7;
    const float alpha = a.alpha != 0.f ? a.alpha : (a.first ? 1.f : 2.f);
    const float* tprev = a.tprev ? a.tprev : a.tp;
    const float* tq = a.tn + 4 * q;
    constexpr int kDotFlush = 16;
    float e0[4], e1[4];
    int since_flush = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) e0[c] = e1[c] = 0.f;
    auto flush = [&]() {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        e0[c] += __shfl_xor_sync(0xffffffffu, e0[c], 8);
        e1[c] += __shfl_xor_sync(0xffffffffu, e1[c], 8);
        e0[c] += __shfl_xor_sync(0xffffffffu, e0[c], 16);
        e1[c] += __shfl_xor_sync(0xffffffffu, e1[c], 16);
      }
      float v0 = 0.f, v1 = 0.f;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float s0 = __shfl_sync(0xffffffffu, e0[c], lane >> 2);
        const float s1 = __shfl_sync(0xffffffffu, e1[c], lane >> 2);
        if ((lane & 3) == c) {
          v0 = s0;
          v1 = s1;
        }
      }
      d0 += (double)v0;
      d1 += (double)v1;
#pragma unroll
      for (int c = 0; c < 4; ++c) e0[c] = e1[c] = 0.f;
    };

    bool gave_up = false;
    if (a.never_wait && !bounded_wait(&never, 0u, a.spin_limit)) {
      if (lane == 0) atomicExch(a.status, leo2d::kStatusTimeout);
      gave_up = true;
    }
    for (int it = 0; !gave_up; ++it) {
      const int64_t tile = tile_of(it);
      if (tile >= n_tiles) break;
      const int stage = it % nst;
      if (!bounded_wait(&full[stage], (uint32_t)(it / nst) & 1u, a.spin_limit)) {
        if (lane == 0) atomicExch(a.status, leo2d::kStatusTimeout);
        break;
      }
      const unsigned char* st = smem + (size_t)stage * a.stage_bytes;
      const int64_t* off_s = reinterpret_cast<const int64_t*>(st);
      const unsigned char* win = st + a.off_bytes + a.data_bytes;
      const int64_t b0 = tile * TB;
      const int64_t ba = b0 & ~1ll;
      const int64_t rb = b0 + warp;
      if (rb < a.nrb) {
        const int64_t sb = off_s[rb - ba];
        const int K = (int)(off_s[rb + 1 - ba] - sb);
        const unsigned char* base = st + a.off_bytes + (size_t)(sb - off_s[b0 - ba]) * kRbSlotBytes;
        const int32_t* psg = reinterpret_cast<const int32_t*>(base) + g;
        const float4* vsg = reinterpret_cast<const float4*>(base + (size_t)K * 4) + g;
        const unsigned char* wq = win + 16 * q;
        const int64_t row = rb * kRbRows + g;
        const bool ok = row < a.n;
        // epilogue operands first: their latency overlaps the slots
        float4 xn = make_float4(0.f, 0.f, 0.f, 0.f), xp = xn;
        if (ok) {
          xn = ldg4(tq + row * C);
          if (!a.first) xp = ld_once4(tprev + row * C + 4 * q);
        }
        const int nb = K >> 2;
        PanelAcc<PACKED> acc;
        acc.zero();
        int b = 0;
        for (; b + U <= nb; b += U) {
          const int32_t* pb = psg + 4 * b;
          const float4* vb = vsg + 4 * b;
          float4 x[U];
#pragma unroll
          for (int u = 0; u < U; ++u) x[u] = *reinterpret_cast<const float4*>(wq + (size_t)pb[4 * u] * 128);
#pragma unroll
          for (int u = 0; u < U; ++u) acc.add(x[u], vb[4 * u]);
        }
        for (; b < nb; ++b) acc.add(*reinterpret_cast<const float4*>(wq + (size_t)psg[4 * b] * 128), vsg[4 * b]);
        float p[4][4];
        acc.get(p);
        const bool upper = g >= 2, odd = (g & 1) != 0;
        float hh[2][4];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const float send = upper ? p[i][c] : p[2 + i][c];
            const float keep = upper ? p[2 + i][c] : p[i][c];
            hh[i][c] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
          }
        float h[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float send = odd ? hh[0][c] : hh[1][c];
          const float keep = odd ? hh[1][c] : hh[0][c];
          h[c] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
        }
        if (ok) {
          float4 y;
          if (a.first) {
            y = make_float4(alpha * h[0], alpha * h[1], alpha * h[2], alpha * h[3]);
          } else {
            y = make_float4(alpha * h[0] - xp.x, alpha * h[1] - xp.y, alpha * h[2] - xp.z, alpha * h[3] - xp.w);
          }
          *reinterpret_cast<float4*>(a.tp + row * C + 4 * q) = y;
          e0[0] += xn.x * xn.x;
          e0[1] += xn.y * xn.y;
          e0[2] += xn.z * xn.z;
          e0[3] += xn.w * xn.w;
          e1[0] += y.x * xn.x;
          e1[1] += y.y * xn.y;
          e1[2] += y.z * xn.z;
          e1[3] += y.w * xn.w;
        }
        if (++since_flush == kDotFlush) {
          since_flush = 0;
          flush();
        }
      }
      // release the stage to the producer
      __syncwarp();
      if (lane == 0) mbar_arrive_cta(&empty[stage]);
    }
    flush();
  }
  __syncthreads();
  // copies in flight (after a timeout) land before the block exits
  if (threadIdx.x == 0)
    for (int i = 0; i < nst; ++i)
      if (issued[i] > 0) bounded_wait(&full[i], (uint32_t)(issued[i] - 1) & 1u, ~0ull);

  __shared__ double bsum[2 * C];
  for (int t = threadIdx.x; t < 2 * C; t += NT) bsum[t] = 0.0;
  __syncthreads();
  for (int w = 0; w < TB; ++w) {
    if (warp == w) {
      bsum[2 * lane] += d0;
      bsum[2 * lane + 1] += d1;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < 2 * C; t += NT) a.partials[(size_t)bid * 2 * C + t] = bsum[t];
}

int rbw_off_bytes() { return ((kRbwTile + 4) * 8 + 127) / 128 * 128; }

}  // namespace

namespace leo2d {

void csr_drop_rbw(leo2d_csr* csr) {
  csr->rbw_built = false;
  csr->rbw_tiles = 0;
  csr->rbw_max_win = 0;
  csr->rbw_tile_max_bytes = 0;
  csr->rbw_roff.release();
  csr->rbw_runs.release();
  csr->rbw_wrows.release();
  csr->rbw_data.release();
}

bool csr_build_rbw(leo2d_ctx* ctx, leo2d_csr* csr) {
  LEO_REQUIRE(csr->rb_built, "windows are built from the row blocks");
  csr_drop_rbw(csr);
  const int64_t nrb = csr->rb_blocks;
  const int64_t tiles = (nrb + kRbwTile - 1) / kRbwTile;
  DevBuf<int64_t> cnt((size_t)tiles);
  csr->rbw_roff.alloc((size_t)tiles + 1);
  csr->rbw_wrows.alloc((size_t)tiles);
  DevBuf<int> err(2);
  DevBuf<unsigned long long> wsum(1);
  LEO_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), ctx->stream));
  LEO_CUDA(cudaMemsetAsync(wsum.p, 0, sizeof(unsigned long long), ctx->stream));
  const size_t smem = (size_t)(kRbwMaxSlots + 2 * kRbwMaxWin + kRbwMaxRuns) * sizeof(uint32_t);
  LEO_CUDA(cudaFuncSetAttribute(k_rbw_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, (int64_t)ctx->sm_count * 4);
  launch(ctx, "rbw_build", [&] {
    k_rbw_build<<<grid, kRbwBuildThreads, smem, ctx->stream>>>(nrb, kRbwTile, csr->rb_off.p, csr->rb_data.p, 0, cnt.p,
                                                                csr->rbw_wrows.p, nullptr, nullptr, nullptr, err.p,
                                                                wsum.p);
  });
  int h[2] = {0, 0};
  unsigned long long ws = 0;
  d2h(ctx, h, err.p, 2);
  d2h(ctx, &ws, wsum.p, 1);
  ctx_sync(ctx);
  if (h[0] != 0) {
    csr_drop_rbw(csr);
    return false;
  }
  exclusive_scan_i64(ctx, cnt.p, csr->rbw_roff.p, tiles);
  int64_t total = 0;
  d2h(ctx, &total, csr->rbw_roff.p + tiles, 1);
  ctx_sync(ctx);
  csr->rbw_runs.alloc((size_t)std::max<int64_t>(2 * total, 2));
  const size_t data_bytes = (size_t)std::max<int64_t>(csr->rb_slots, 1) * kRbSlotBytes;
  csr->rbw_data.alloc(data_bytes);
  LEO_CUDA(cudaMemcpyAsync(csr->rbw_data.p, csr->rb_data.p, data_bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  launch(ctx, "rbw_build", [&] {
    k_rbw_build<<<grid, kRbwBuildThreads, smem, ctx->stream>>>(nrb, kRbwTile, csr->rb_off.p, csr->rb_data.p, 1,
                                                                nullptr, nullptr, csr->rbw_roff.p, csr->rbw_runs.p,
                                                                csr->rbw_data.p, err.p, wsum.p);
  });
  ctx_sync(ctx);
  csr->rbw_tiles = tiles;
  csr->rbw_tile_max_bytes = rb_tile_max_bytes(ctx, csr, kRbwTile);
  csr->rbw_max_win = h[1];
  csr->rbw_win_rows = (int64_t)ws;
  csr->rbw_runs_total = total;
  csr->rbw_built = true;
  return true;
}

// Bytes of one stage: offsets, the largest tile's slots, the widest window.
static int64_t rbw_stage_bytes(const leo2d_csr* csr) {
  const int64_t data = (csr->rbw_tile_max_bytes + 127) / 128 * 128;
  return rbw_off_bytes() + data + (int64_t)csr->rbw_max_win * 128;
}

int rbw_stages(leo2d_ctx* ctx, leo2d_csr* csr) {
  if (!csr->rbw_built) return 0;
  const int64_t stage = rbw_stage_bytes(csr);
  const int64_t budget = (int64_t)ctx->smem_optin - 6 * 1024;  // static shared memory of the kernel (~5 KB)
  const int64_t s = std::min<int64_t>(4, budget / std::max<int64_t>(stage, 1));
  return s >= 2 ? (int)std::min<int64_t>(s, std::max(2, ctx->tile_stages)) : 0;
}

size_t rbw_smem_bytes(leo2d_ctx* ctx, leo2d_csr* csr) {
  return (size_t)rbw_stages(ctx, csr) * (size_t)rbw_stage_bytes(csr);
}

unsigned rbw_grid(leo2d_ctx* ctx, const leo2d_csr* csr) {
  const int64_t chunks = (csr->rbw_tiles + ctx->tile_chunk - 1) / std::max(1, ctx->tile_chunk);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->sm_count, chunks));
}

void rbw_launch_step(leo2d_ctx* ctx, const leo2d_csr* csr, const StepShape& shape, unsigned grid, size_t smem,
                     const float* tn, float* tp, const float* tprev, int first, float alpha, double* partials,
                     const double* prev_partials, double* prev_dots) {
  leo2d_csr* m = const_cast<leo2d_csr*>(csr);
  RbwArgs a{};
  a.n = csr->n;
  a.nrb = csr->rb_blocks;
  a.off = csr->rb_off.p;
  a.data = csr->rbw_data.p;
  a.roff = csr->rbw_roff.p;
  a.runs = csr->rbw_runs.p;
  a.wrows = csr->rbw_wrows.p;
  a.tn = tn;
  a.tp = tp;
  a.tprev = tprev;
  a.first = first;
  a.alpha = alpha;
  a.partials = partials;
  a.prev_partials = prev_partials;
  a.prev_dots = prev_dots;
  a.stages = rbw_stages(ctx, m);
  LEO_REQUIRE(a.stages >= 2, "row-block windows too large for shared memory");
  a.chunk = std::max(1, ctx->tile_chunk);
  a.off_bytes = rbw_off_bytes();
  a.data_bytes = (int)((csr->rbw_tile_max_bytes + 127) / 128 * 128);
  a.stage_bytes = (int)rbw_stage_bytes(m);
  LEO_REQUIRE((size_t)a.stages * a.stage_bytes <= smem, "row-block shared memory changed since setup");
  a.spin_limit = ctx->spin_limit;
  a.status = ctx->status.p;
  a.never_wait = ctx->test_unsatisfied_wait;
  auto go = [&](auto kern) {
    LEO_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    launch(ctx, "cheb_step", [&] { kern<<<grid, (kRbwTile + 1) * 32, smem, ctx->stream>>>(a); });
  };
  const bool u8 = shape.rb_unroll == 8;
  if (shape.rb_packed) {
    if (u8) return go(k_cheb_rbw<kRbwTile, true, 8>);
    return go(k_cheb_rbw<kRbwTile, true, 4>);
  }
  if (u8) return go(k_cheb_rbw<kRbwTile, false, 8>);
  return go(k_cheb_rbw<kRbwTile, false, 4>);
}

}  // namespace leo2d
