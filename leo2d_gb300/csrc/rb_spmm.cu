// rb_spmm.cu - the row-block Chebyshev step (FP32, 32 columns).
//
// Same step as the tiled CSR kernel (T_{n+1} = a H~ T_n - T_{n-1} with the two
// moment dots fused; Locality::computeDosTraceKPM, src/locality.cpp:6195-6234),
// over a second layout of the locality-ordered matrix that removes its
// bottleneck: the CSR step gathers one 128-byte T_n row per stored entry
// (about 65 per row for twisted bilayers), and the L1 data pipe that serves
// those gathers, not HBM, bounds it.
//
// Row-block format (built once per matrix from the locality-ordered copy):
// rows are taken in blocks of 4 consecutive rows; a row block stores the sorted
// union of its rows' columns (its slots) and a dense 4 x slots panel of values
// (zero where a row has no entry). One gather of a T_n row serves the 4 rows:
// with the patch ordering, 4 rows share most of their neighbours, so a block
// holds about 26 slots per row against 65 entries, and the stream is 20 bytes
// per slot against 8 per entry.
//
// Layout in HBM
//   rb_off   int64[nrb + 1 (+pad)]  first slot of each row block; multiples of 4
//   rb_data  row block b at byte 20 * rb_off[b], K = rb_off[b+1] - rb_off[b] slots:
//              int32 col[K]          (slots past the union are padding: a valid
//                                     column with zero values)
//              float val[K][4]       value of row r of the block at slot s
// Kernel (one block per SM, WARPS warps)
//   An elected lane copies tiles of WARPS row blocks (their offsets and data)
//   into a 2..4-stage shared-memory ring with cp.async.bulk, completing on
//   mbarriers; warp w takes row block w of each tile. Slots go in batches of
//   four: group g (lanes 8g..8g+7) takes slot 4b + g and lane q of the group
//   columns 4q..4q+3, so each quarter-warp gathers one whole 128-byte T_n row:
//   one L1 wavefront per slot (a 16-byte load is served a quarter-warp at a
//   time, so four groups reading the same row would cost four). The lane reads
//   the slot's 4 values with one 16-byte shared load and accumulates the 4 rows
//   over its 4 columns; a shuffle reduce-scatter over the groups leaves row g
//   with group g. Epilogue, dots and the fixed-order partials are those of the
//   CSR kernels. Every wait is bounded (two seconds or the context's poll
//   limit) and reports a status.
#include <algorithm>
#include <cstring>
#include <cmath>

#include "kpm.cuh"

using namespace leo2d;

#include "step_kernels.cuh"

namespace {

#include "rb_common.cuh"

constexpr int kRbBuildThreads = 256;
constexpr int kRbMaxEnt = 4096;     // stored entries of one row block (build limit)
constexpr int kRbMaxSlots = 2048;   // slots of one row block (build limit)
constexpr int kRbOffPad = 8;        // int64 elements past off[nrb] (tile copies round their range up)

struct RbArgs {
  int64_t n;    // rows
  int64_t nrb;  // row blocks
  const int64_t* __restrict__ off;
  const unsigned char* __restrict__ data;
  const float* __restrict__ tn;
  float* __restrict__ tp;
  const float* __restrict__ tprev;  // null: T_{n-1} is read from tp
  int first;
  float alpha;  // 0: the default (1 for the first step, else 2)
  double* __restrict__ partials;
  const double* __restrict__ prev_partials;
  double* __restrict__ prev_dots;
  const float* __restrict__ im;  // complex H: [slots][4] imaginary panel
  // velocity mode: x of each row and of each slot's column relative to the
  // block's first row ([blocks][4] and [slots]), and the output for D T_n,
  // D_ij = (x_i - x_j) H~_ij
  const float* __restrict__ xrel;
  const float* __restrict__ xs;
  float* __restrict__ out2;
  int stages;      // 2..4
  int chunk;       // consecutive tiles per block between grid-wide jumps
  int off_bytes;   // offsets region of a stage
  int panel_at;    // start of the second panel in a stage (complex H: imaginary values; velocity: x)
  int stage_bytes; // offsets + data (+ imaginary panel), multiple of 128
  uint64_t spin_limit;
  int* status;
  int never_wait;  // test hook: wait on a barrier that nobody completes
};

// One CTA's share of a step: CTA `bid` of `nblk` working on the matrix of `a`
// (the whole grid for one matrix, a block group of a batched launch).
template <int WARPS, bool PACKED, int U, bool CPX = false, bool DJ = false>
__device__ __forceinline__ void rb_body(const RbArgs& a, const int bid, const int nblk) {
  constexpr int C = 32;
  constexpr int NT = WARPS * 32;
  constexpr int kMaxStages = 4;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kMaxStages];
  __shared__ int released[kMaxStages];
  __shared__ int issued[kMaxStages];
  __shared__ __align__(8) uint64_t never;
  if (a.prev_partials) reduce_prev<C, NT>(a.prev_partials, a.prev_dots, nblk, bid, nblk);

  const int nst = a.stages;
  const int64_t n_tiles = (a.nrb + WARPS - 1) / WARPS;
  if (threadIdx.x == 0) {
    for (int i = 0; i < nst; ++i) {
      mbar_init(&full[i], 1);
      released[i] = 0;
      issued[i] = 0;
    }
    mbar_init(&never, 1);
    mbar_fence_init();
  }
  __syncthreads();

  // copies of `tile` (its offsets, rounded out to 16 bytes, and its data) into `stage`
  auto issue = [&](int64_t tile, int stage) {
    const int64_t b0 = tile * WARPS, b1 = min(a.nrb, b0 + WARPS);
    const int64_t ba = b0 & ~1ll;
    const int64_t ocount = ((b1 + 1 - ba) + 1) & ~1ll;
    const int64_t s0 = a.off[b0], s1 = a.off[b1];
    const uint32_t dbytes = (uint32_t)((s1 - s0) * kRbSlotBytes);
    unsigned char* st = smem + (size_t)stage * a.stage_bytes;
    const uint32_t ibytes = CPX  ? (uint32_t)((s1 - s0) * kRbRows * sizeof(float))
                            : DJ ? (uint32_t)((s1 - s0) * sizeof(float))
                                 : 0u;
    issued[stage] += 1;
    mbar_expect_tx(&full[stage], (uint32_t)(ocount * 8) + dbytes + ibytes);
    bulk_g2s(st, a.off + ba, (uint32_t)(ocount * 8), &full[stage]);
    if (dbytes) bulk_g2s(st + a.off_bytes, a.data + s0 * kRbSlotBytes, dbytes, &full[stage]);
    if (CPX && ibytes) bulk_g2s(st + a.panel_at, a.im + s0 * kRbRows, ibytes, &full[stage]);
    if (DJ && ibytes) bulk_g2s(st + a.panel_at, a.xs + s0, ibytes, &full[stage]);
  };
  const int64_t chunk = a.chunk;
  auto tile_of = [&](int64_t i) -> int64_t {
    return ((int64_t)bid + (i / chunk) * (int64_t)nblk) * chunk + i % chunk;
  };
  if (threadIdx.x == 0)
    for (int i = 0; i < nst; ++i)
      if (tile_of(i) < n_tiles) issue(tile_of(i), i);
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 3, q = lane & 7;
  const float alpha = a.alpha != 0.f ? a.alpha : (a.first ? 1.f : 2.f);
  const float* tprev = a.tprev ? a.tprev : a.tp;
  const float* tq = a.tn + 4 * q;
  // dots: FP32 over kDotFlush row blocks (64 rows), then FP64 (the FP64 pipe
  // is a small fraction of the FP32 one: converting every block's partials
  // would bound the kernel). A flush sums the four groups' FP32 partials and
  // hands column `lane` to lane `lane`, so the FP64 sums take 2 registers.
  constexpr int kDotFlush = 16;
  double d0 = 0.0, d1 = 0.0;  // column `lane`
  float e0[4], e1[4];         // columns 4q..4q+3, this lane's rows
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
    // column `lane` = 4 * (lane >> 2) + (lane & 3) lives in lane (lane >> 2)
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

  int it = 0;
  for (int64_t tile = tile_of(0); !gave_up && tile < n_tiles; tile = tile_of(++it)) {
    const int stage = it % nst;
    const uint32_t parity = (uint32_t)(it / nst) & 1u;
    if (!bounded_wait(&full[stage], parity, a.spin_limit)) {
      if (lane == 0) atomicExch(a.status, leo2d::kStatusTimeout);
      break;
    }
    const unsigned char* st = smem + (size_t)stage * a.stage_bytes;
    const int64_t* off_s = reinterpret_cast<const int64_t*>(st);
    const int64_t b0 = tile * WARPS;
    const int64_t ba = b0 & ~1ll;
    const int64_t rb = b0 + warp;
    if (rb < a.nrb) {
      const int64_t sb = off_s[rb - ba];
      const int K = (int)(off_s[rb + 1 - ba] - sb);
      const unsigned char* base = st + a.off_bytes + (size_t)(sb - off_s[b0 - ba]) * kRbSlotBytes;
      const int32_t* cs = reinterpret_cast<const int32_t*>(base);
      const float4* vs = reinterpret_cast<const float4*>(base + (size_t)K * 4);
      const int64_t row = rb * kRbRows + g;
      const bool ok = row < a.n;
      // the epilogue's rows, fetched into L1 while the slots run
      if (ok) {
        if (!DJ) asm volatile("prefetch.global.L1 [%0];" ::"l"(tq + row * C));
        if (!a.first) asm volatile("prefetch.global.L1 [%0];" ::"l"(tprev + row * C + 4 * q));
      }
      // batches of 4 slots, U batches in flight per lane; the main loop runs
      // whole groups of U batches at fixed offsets, the rest in guarded groups of 4
      const int nb = K >> 2;
      const int32_t* csg = cs + g;
      const float4* vsg = vs + g;
      const float4* wsg = reinterpret_cast<const float4*>(st + a.panel_at) + (sb - off_s[b0 - ba]) + g;
      const float* xsg = reinterpret_cast<const float*>(st + a.panel_at) + (sb - off_s[b0 - ba]) + g;
      typename std::conditional<CPX, PanelAccCpx, PanelAcc<PACKED>>::type acc;
      acc.zero();
      // velocity mode: a second accumulator for D T_n, D_ij = (x_i - x_j) H~_ij
      // built on the fly from positions relative to the block's first row (FP64
      // differences rounded once: small numbers, so x_i - x_j keeps the FP32
      // accuracy of the difference itself)
      PanelAcc<PACKED> accj;
      float4 xr;
      if constexpr (DJ) {
        accj.zero();
        xr = __ldg(reinterpret_cast<const float4*>(a.xrel) + rb);
      }
      auto add = [&](const float4& x, int slot4) {
        if constexpr (CPX) {
          acc.add(x, vsg[slot4], wsg[slot4]);
        } else {
          const float4 v = vsg[slot4];
          acc.add(x, v);
          if constexpr (DJ) {
            const float e = xsg[slot4];
            accj.add(x, make_float4(v.x * (xr.x - e), v.y * (xr.y - e), v.z * (xr.z - e), v.w * (xr.w - e)));
          }
        }
      };
      int b = 0;
      for (; b + U <= nb; b += U) {
        const int32_t* cb = csg + 4 * b;
        const float4* vb = vsg + 4 * b;
        uint32_t c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) c[u] = (uint32_t)cb[4 * u];
        float4 x[U];
#pragma unroll
        for (int u = 0; u < U; ++u) x[u] = ldg4(tq + (size_t)c[u] * C);
#pragma unroll
        for (int u = 0; u < U; ++u) add(x[u], 4 * (b + u));
        (void)vb;
      }
      for (; b < nb; b += 4) {
        const int rem = nb - b;  // warp-uniform
        const int32_t* cb = csg + 4 * b;
        const float4* vb = vsg + 4 * b;
        float4 x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          x[u] = u < rem ? ldg4(tq + (size_t)(uint32_t)cb[4 * u] * C) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (u < rem) add(x[u], 4 * (b + u));
        (void)vb;
      }
      // reduce-scatter over the four groups: group g keeps row g
      const bool upper = g >= 2, odd = (g & 1) != 0;
      auto scatter = [&](const float (&p)[4][4], float (&h)[4]) {
        float hh[2][4];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const float send = upper ? p[i][c] : p[2 + i][c];
            const float keep = upper ? p[2 + i][c] : p[i][c];
            hh[i][c] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
          }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float send = odd ? hh[0][c] : hh[1][c];
          const float keep = odd ? hh[1][c] : hh[0][c];
          h[c] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
        }
      };
      float h[4];
      {
        float p[4][4];
        acc.get(p);
        scatter(p, h);
      }
      if constexpr (DJ) {
        float p[4][4], hj[4];
        accj.get(p);
        scatter(p, hj);
        if (ok) st_na4(a.out2 + row * C + 4 * q, make_float4(hj[0], hj[1], hj[2], hj[3]));
      }
      if (ok) {
        float4 y;
        if (a.first) {
          y = make_float4(alpha * h[0], alpha * h[1], alpha * h[2], alpha * h[3]);
        } else {
          const float4 xp = ldcs4(tprev + row * C + 4 * q);
          y = make_float4(alpha * h[0] - xp.x, alpha * h[1] - xp.y, alpha * h[2] - xp.z, alpha * h[3] - xp.w);
        }
        st_na4(a.tp + row * C + 4 * q, y);
        if constexpr (!DJ) {
          const float4 xn = ldg4(tq + row * C);
          e0[0] += xn.x * xn.x;
          e0[1] += xn.y * xn.y;
          e0[2] += xn.z * xn.z;
          e0[3] += xn.w * xn.w;
          e1[0] += y.x * xn.x;
          e1[1] += y.y * xn.y;
          e1[2] += y.z * xn.z;
          e1[3] += y.w * xn.w;
        }
      }
      if constexpr (!DJ) {
        if (++since_flush == kDotFlush) {  // warp-uniform
          since_flush = 0;
          flush();
        }
      }
    }
    // release the stage; the last warp refills it
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      if (atomicAdd(&released[stage], 1) == WARPS - 1) {
        released[stage] = 0;
        const int64_t nt = tile_of(it + nst);
        if (nt < n_tiles) issue(nt, stage);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  // a copy may still be in flight after a timeout: it lands before the block exits
  if (threadIdx.x == 0)
    for (int i = 0; i < nst; ++i)
      if (issued[i] > 0) bounded_wait(&full[i], (uint32_t)(issued[i] - 1) & 1u, ~0ull);

  // (the velocity step computes no moment dots and writes no partials)
  if constexpr (DJ) return;
  flush();
  // warps add their columns in warp order (deterministic)
  __shared__ double bsum[2 * C];
  for (int t = threadIdx.x; t < 2 * C; t += NT) bsum[t] = 0.0;
  __syncthreads();
  for (int w = 0; w < WARPS; ++w) {
    if (warp == w) {
      bsum[2 * lane] += d0;
      bsum[2 * lane + 1] += d1;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < 2 * C; t += NT) a.partials[(size_t)bid * 2 * C + t] = bsum[t];
}

template <int WARPS, bool PACKED, int U, bool CPX = false, bool DJ = false>
__global__ void __launch_bounds__(WARPS * 32, 1) k_cheb_rb(const __grid_constant__ RbArgs a) {
  rb_body<WARPS, PACKED, U, CPX, DJ>(a, (int)blockIdx.x, (int)gridDim.x);
}

// Several matrices in one launch: matrix f runs on the CTAs [block_first[f],
// block_first[f+1]) as block group of its own (tiles, partials and the deferred
// reduction stay within the matrix).
struct RbBatchParams {
  RbArgs f[kRbBatchMax];
  int block_first[kRbBatchMax + 1];
  int nflakes;
};
static_assert(sizeof(RbBatchParams) <= 32764, "batched row-block parameters exceed the parameter space");

template <int WARPS, bool PACKED, int U>
__global__ void __launch_bounds__(WARPS * 32, 1) k_cheb_rb_batch(const __grid_constant__ RbBatchParams p) {
  int f = 0;
  while (f + 1 < p.nflakes && (int)blockIdx.x >= p.block_first[f + 1]) ++f;
  rb_body<WARPS, PACKED, U>(p.f[f], (int)blockIdx.x - p.block_first[f], p.block_first[f + 1] - p.block_first[f]);
}

// ---------------------------------------------------------------- format build

// Positions for the velocity step, relative to each row block's first row and
// rounded once from the FP64 difference: xrel[4b + k] = x(row 4b + k) - x(row 4b)
// (0 past the last row), xs[s] = x(column of slot s) - x(row 4b) (one warp per
// row block; rows and columns in the ordered numbering).
__global__ void k_rb_xrel(int64_t n, int64_t nrb, const int64_t* __restrict__ off,
                          const unsigned char* __restrict__ data, const double* __restrict__ pos,
                          const int32_t* __restrict__ new2old, float* __restrict__ xrel, float* __restrict__ xs) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < nrb; b += warps) {
    const double x0 = pos[3 * (int64_t)new2old[b * kRbRows]];
    if (lane < kRbRows) {
      const int64_t r = b * kRbRows + lane;
      xrel[r] = r < n ? (float)(pos[3 * (int64_t)new2old[r]] - x0) : 0.f;
    }
    const int64_t s0 = off[b];
    const int K = (int)(off[b + 1] - s0);
    const int32_t* col = reinterpret_cast<const int32_t*>(data + s0 * kRbSlotBytes);
    for (int k = lane; k < K; k += 32) xs[s0 + k] = (float)(pos[3 * (int64_t)new2old[col[k]]] - x0);
  }
}

// Ascending bitonic sort of n (a power of two >= blockDim.x) keys in shared memory.
__device__ void bitonic_sort_u64(unsigned long long* key, int n) {
  for (int k = 2; k <= n; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool up = (i & k) == 0;
          const unsigned long long x = key[i], y = key[ixj];
          if ((x > y) == up) {
            key[i] = y;
            key[ixj] = x;
          }
        }
      }
      __syncthreads();
    }
}

// Exclusive prefix sum of one int per thread over the block; *total gets the sum.
__device__ int rb_block_scan(int x, int* total) {
  __shared__ int s[kRbBuildThreads];
  s[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < kRbBuildThreads; o <<= 1) {
    const int v = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  const int incl = s[threadIdx.x];
  *total = s[kRbBuildThreads - 1];
  __syncthreads();
  return incl - x;
}

constexpr int kRbWarpCap = 512;     // entries of a row block the warp-per-block build sorts
constexpr int kRbWarpsPerCta = 8;

// The same two passes with one warp per row block, for blocks of at most
// kRbWarpCap entries (a twisted bilayer's 4 rows hold about 260), with warp
// barriers only: pass 0 counts the distinct columns in a hash set, pass 1 sorts
// the keys in the warp's slice of shared memory. Larger blocks are appended to
// `big` in pass 0 and left to k_rb_build.
__global__ void __launch_bounds__(kRbWarpsPerCta * 32)
    k_rb_build_warp(int64_t n, int64_t nrb, const int64_t* __restrict__ prow, const int32_t* __restrict__ pcol,
                    const float* __restrict__ pval, const float* __restrict__ pval_im, int pass,
                    int64_t* __restrict__ count, const int64_t* __restrict__ off, unsigned char* __restrict__ data,
                    float* __restrict__ im_out, int* __restrict__ err, unsigned long long* __restrict__ ssum,
                    int64_t* __restrict__ big, unsigned long long* __restrict__ n_big) {
  __shared__ unsigned long long keys_all[kRbWarpsPerCta][kRbWarpCap];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long* keys = keys_all[w];
  const int64_t warps = (int64_t)gridDim.x * kRbWarpsPerCta;
  for (int64_t b = (int64_t)blockIdx.x * kRbWarpsPerCta + w; b < nrb; b += warps) {
    const int64_t r0 = b * kRbRows;
    const int rows = (int)min((int64_t)kRbRows, n - r0);
    const int64_t mine = lane <= kRbRows ? prow[r0 + min(lane, rows)] : 0;
    int64_t srp[kRbRows + 1];
#pragma unroll
    for (int k = 0; k <= kRbRows; ++k) srp[k] = __shfl_sync(0xffffffffu, mine, k);
    // srp[k] with k in registers (a run-time index would put srp in local memory)
    auto srp_at = [&](int k) {
      int64_t v = srp[0];
#pragma unroll
      for (int kk = 1; kk <= kRbRows; ++kk)
        if (k == kk) v = srp[kk];
      return v;
    };
    const int64_t q0 = srp[0];
    const int E = (int)(srp_at(rows) - q0);
    if (E > kRbWarpCap) {
      if (pass == 0 && lane == 0) big[atomicAdd(n_big, 1ull)] = b;
      continue;
    }
    __syncwarp();  // the previous block's keys are read
    if (pass == 0) {
      // counting needs the distinct columns only: a hash set in the warp's slice
      // (2 x kRbWarpCap 32-bit slots, load <= 1/2), no sort
      uint32_t* set = reinterpret_cast<uint32_t*>(keys);
      constexpr int kSet = 2 * kRbWarpCap;
      for (int i = lane; i < kSet; i += 32) set[i] = 0xFFFFFFFFu;
      __syncwarp();
      int fresh = 0;
      for (int i = lane; i < E; i += 32) {
        const uint32_t c = (uint32_t)pcol[q0 + i];
        uint32_t h = (c * 2654435761u) & (kSet - 1);
        for (int probe = 0; probe < kSet; ++probe) {  // bounded: the set never fills
          const uint32_t prev = atomicCAS(&set[h], 0xFFFFFFFFu, c);
          if (prev == 0xFFFFFFFFu) {
            ++fresh;
            break;
          }
          if (prev == c) break;
          h = (h + 1) & (kSet - 1);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) fresh += __shfl_xor_sync(0xffffffffu, fresh, o);
      if (lane == 0) {
        const int K = fresh, Kp = (K + 3) & ~3;
        if (Kp > kRbMaxSlots) atomicOr(&err[0], 2);
        count[b] = Kp;
        atomicMax(&err[1], K);
        atomicAdd(ssum, (unsigned long long)K);
      }
      continue;
    }
    int P2 = 32;
    while (P2 < E) P2 <<= 1;
    for (int i = lane; i < P2; i += 32)
      keys[i] = i < E ? (((unsigned long long)(uint32_t)pcol[q0 + i] << 16) | (unsigned long long)i) : ~0ull;
    __syncwarp();
    for (int k = 2; k <= P2; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < P2; i += 32) {
          const int ixj = i ^ j;
          if (ixj > i) {
            const bool up = (i & k) == 0;
            const unsigned long long x = keys[i], y = keys[ixj];
            if ((x > y) == up) {
              keys[i] = y;
              keys[ixj] = x;
            }
          }
        }
        __syncwarp();
      }
    // slot of each sorted entry: distinct columns counted in order
    const int per = P2 / 32;
    const int i0 = lane * per;
    int cnt = 0;
    for (int j = 0; j < per; ++j) {
      const int i = i0 + j;
      if (i < E && (i == 0 || (keys[i] >> 16) != (keys[i - 1] >> 16))) ++cnt;
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int K = __shfl_sync(0xffffffffu, incl, 31);
    const int first_slot = incl - cnt;
    const int Kp = (K + 3) & ~3;
    int32_t* col_out = reinterpret_cast<int32_t*>(data + off[b] * kRbSlotBytes);
    float* val_out = reinterpret_cast<float*>(data + off[b] * kRbSlotBytes + (size_t)Kp * 4);
    for (int i = lane; i < Kp * kRbRows; i += 32) val_out[i] = 0.f;
    const int32_t pad_col = K > 0 ? (int32_t)(keys[0] >> 16) : 0;
    for (int s = K + lane; s < Kp; s += 32) col_out[s] = pad_col;
    __syncwarp();
    int s = first_slot - 1;
    for (int j = 0; j < per; ++j) {
      const int i = i0 + j;
      if (i >= E) break;
      const unsigned long long k = keys[i];
      const uint32_t c = (uint32_t)(k >> 16);
      const int e = (int)(k & 0xFFFFu);
      const bool new_col = i == 0 || (keys[i - 1] >> 16) != c;
      if (new_col) {
        ++s;
        col_out[s] = (int32_t)c;
      }
      int r = 0;
#pragma unroll
      for (int k = 1; k < kRbRows; ++k) r += (k < rows && srp[k] - q0 <= e) ? 1 : 0;
      const int64_t row_lo = srp_at(r) - q0, row_hi = srp_at(r + 1) - q0;
      // the first entry of each (column, row) run sums the run in entry order
      bool start = new_col;
      if (!start) {
        const int ep = (int)(keys[i - 1] & 0xFFFFu);
        start = !(row_lo <= ep);
      }
      if (start) {
        float v = pval[q0 + e];
        float vi = pval_im ? pval_im[q0 + e] : 0.f;
        for (int m = i + 1; m < E && (uint32_t)(keys[m] >> 16) == c; ++m) {
          const int em = (int)(keys[m] & 0xFFFFu);
          if (em >= row_hi) break;
          v += pval[q0 + em];
          if (pval_im) vi += pval_im[q0 + em];
        }
        val_out[s * kRbRows + r] = v;
        if (im_out) im_out[(off[b] + s) * kRbRows + r] = vi;
      }
    }
  }
}

// Pass 0: count[b] = slots of row block b (union of its rows' columns, padded
// to a multiple of 4). Pass 1: writes row block b at data + 20 * off[b].
// err[0]: bit 0 a block with more than kRbMaxEnt entries, bit 1 more than
// kRbMaxSlots slots; err[1] most slots (before padding); ssum: sum of slots.
// One block of threads per row block: the row blocks in `list` (n_list of
// them), or every row block when list is null.
__global__ void __launch_bounds__(kRbBuildThreads) k_rb_build(int64_t n, int64_t nrb, const int64_t* __restrict__ prow,
                                                              const int32_t* __restrict__ pcol,
                                                              const float* __restrict__ pval,
                                                              const float* __restrict__ pval_im, int pass,
                                                              int64_t* __restrict__ count,
                                                              const int64_t* __restrict__ off,
                                                              unsigned char* __restrict__ data, float* __restrict__ im_out,
                                                              int* __restrict__ err,
                                                              unsigned long long* __restrict__ ssum,
                                                              const int64_t* __restrict__ list, int64_t n_list) {
  extern __shared__ unsigned long long rb_keys[];  // kRbMaxEnt keys: column << 16 | entry
  __shared__ int64_t srp[kRbRows + 1];
  const int64_t todo = list ? n_list : nrb;
  for (int64_t t = blockIdx.x; t < todo; t += gridDim.x) {
    const int64_t b = list ? list[t] : t;
    const int64_t r0 = b * kRbRows;
    const int rows = (int)min((int64_t)kRbRows, n - r0);
    if (threadIdx.x <= kRbRows) srp[threadIdx.x] = prow[r0 + min((int)threadIdx.x, rows)];
    __syncthreads();
    const int64_t q0 = srp[0];
    const int E = (int)(srp[rows] - q0);
    if (E > kRbMaxEnt) {
      if (threadIdx.x == 0) {
        atomicOr(&err[0], 1);
        if (pass == 0) count[b] = 0;
      }
      __syncthreads();
      continue;
    }
    int P2 = kRbBuildThreads;
    while (P2 < E) P2 <<= 1;
    for (int i = threadIdx.x; i < P2; i += blockDim.x)
      rb_keys[i] = i < E ? (((unsigned long long)(uint32_t)pcol[q0 + i] << 16) | (unsigned long long)i)
                         : ~0ull;
    __syncthreads();
    bitonic_sort_u64(rb_keys, P2);
    // slot of each sorted entry: distinct columns counted in order
    const int per = P2 / kRbBuildThreads;
    const int i0 = threadIdx.x * per;
    int cnt = 0;
    for (int j = 0; j < per; ++j) {
      const int i = i0 + j;
      if (i < E && (i == 0 || (rb_keys[i] >> 16) != (rb_keys[i - 1] >> 16))) ++cnt;
    }
    int K = 0;
    const int first_slot = rb_block_scan(cnt, &K);
    const int Kp = (K + 3) & ~3;
    if (pass == 0) {
      if (threadIdx.x == 0) {
        if (Kp > kRbMaxSlots) atomicOr(&err[0], 2);
        count[b] = Kp;
        atomicMax(&err[1], K);
        atomicAdd(ssum, (unsigned long long)K);
      }
      __syncthreads();
      continue;
    }
    int32_t* col_out = reinterpret_cast<int32_t*>(data + off[b] * kRbSlotBytes);
    float* val_out = reinterpret_cast<float*>(data + off[b] * kRbSlotBytes + (size_t)Kp * 4);
    for (int i = threadIdx.x; i < Kp * kRbRows; i += blockDim.x) val_out[i] = 0.f;
    const int32_t pad_col = K > 0 ? (int32_t)(rb_keys[0] >> 16) : 0;
    for (int s = K + (int)threadIdx.x; s < Kp; s += blockDim.x) col_out[s] = pad_col;
    __syncthreads();
    int s = first_slot - 1;
    for (int j = 0; j < per; ++j) {
      const int i = i0 + j;
      if (i >= E) break;
      const unsigned long long k = rb_keys[i];
      const uint32_t c = (uint32_t)(k >> 16);
      const int e = (int)(k & 0xFFFFu);
      const bool new_col = i == 0 || (rb_keys[i - 1] >> 16) != c;
      if (new_col) {
        ++s;
        col_out[s] = (int32_t)c;
      }
      int r = 0;
      while (r + 1 < rows && srp[r + 1] - q0 <= e) ++r;
      // entries of one (column, row) pair are adjacent (sorted by column, then
      // entry index); the first of each run sums the run in entry order
      bool start = new_col;
      if (!start) {
        const int ep = (int)(rb_keys[i - 1] & 0xFFFFu);
        start = !(srp[r] - q0 <= ep);
      }
      if (start) {
        float v = pval[q0 + e];
        float vi = pval_im ? pval_im[q0 + e] : 0.f;
        for (int m = i + 1; m < E && (uint32_t)(rb_keys[m] >> 16) == c; ++m) {
          const int em = (int)(rb_keys[m] & 0xFFFFu);
          if (em >= srp[r + 1] - q0) break;
          v += pval[q0 + em];
          if (pval_im) vi += pval_im[q0 + em];
        }
        val_out[s * kRbRows + r] = v;
        if (im_out) im_out[(off[b] + s) * kRbRows + r] = vi;
      }
    }
    __syncthreads();
  }
}

// Largest data bytes of a tile of `tile` consecutive row blocks.
__global__ void k_rb_tile_max(const int64_t* __restrict__ off, int64_t nrb, int tile,
                              unsigned long long* __restrict__ out) {
  const int64_t tiles = (nrb + tile - 1) / tile;
  unsigned long long m = 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tiles;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = t * tile, b1 = min(nrb, b0 + tile);
    const unsigned long long v = (unsigned long long)(off[b1] - off[b0]) * kRbSlotBytes;
    m = v > m ? v : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, m, o);
    m = y > m ? y : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Offsets region of a stage: (warps + 3) int64 values rounded up to 128 bytes.
int rb_off_bytes(int warps) { return ((warps + 4) * 8 + 127) / 128 * 128; }

// Largest tile (data bytes) for tiles of `warps` row blocks (cached per width).
int64_t rb_tile_bytes(leo2d_ctx* ctx, leo2d_csr* csr, int warps) {
  const bool slot = warps % 8 == 0 && warps >= 8 && warps <= 32;
  if (slot && csr->rb_tile_bytes_w[warps / 8] > 0) {
    csr->rb_tile_warps = warps;
    csr->rb_tile_max_bytes = csr->rb_tile_bytes_w[warps / 8];
    return csr->rb_tile_max_bytes;
  }
  if (csr->rb_tile_warps == warps) return csr->rb_tile_max_bytes;
  DevBuf<unsigned long long> mx(1);
  LEO_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), ctx->stream));
  const int64_t tiles = (csr->rb_blocks + warps - 1) / warps;
  launch(ctx, "rb_tile_max", [&] {
    k_rb_tile_max<<<grid_for(tiles, 256, (int64_t)ctx->sm_count * 8), 256, 0, ctx->stream>>>(
        csr->rb_off.p, csr->rb_blocks, warps, mx.p);
  });
  unsigned long long hm = 0;
  d2h(ctx, &hm, mx.p, 1);
  ctx_sync(ctx);
  csr->rb_tile_warps = warps;
  csr->rb_tile_max_bytes = (int64_t)hm;
  if (slot) csr->rb_tile_bytes_w[warps / 8] = (int64_t)hm;
  return csr->rb_tile_max_bytes;
}

// Imaginary panel of the largest tile (complex H): 16 of every 20 slot bytes.
// Bytes of a stage's second panel: the imaginary values (complex H, 16 per
// slot) or the slots' column positions (velocity step, 4 per slot).
int64_t rb_panel_bytes(leo2d_ctx* ctx, leo2d_csr* csr, int warps, bool velocity) {
  const int64_t per = velocity ? (int64_t)sizeof(float) : (csr->complex_h ? kRbRows * (int64_t)sizeof(float) : 0);
  if (per == 0) return 0;
  return (rb_tile_bytes(ctx, csr, warps) / kRbSlotBytes * per + 127) / 128 * 128;
}

int64_t rb_stage_bytes(leo2d_ctx* ctx, leo2d_csr* csr, int warps, bool velocity) {
  return rb_off_bytes(warps) + (rb_tile_bytes(ctx, csr, warps) + 127) / 128 * 128 +
         rb_panel_bytes(ctx, csr, warps, velocity);
}

}  // namespace

namespace leo2d {

int64_t rb_tile_max_bytes(leo2d_ctx* ctx, const leo2d_csr* csr, int tile) {
  DevBuf<unsigned long long> mx(1);
  LEO_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), ctx->stream));
  const int64_t tiles = (csr->rb_blocks + tile - 1) / tile;
  launch(ctx, "rb_tile_max", [&] {
    k_rb_tile_max<<<grid_for(tiles, 256, (int64_t)ctx->sm_count * 8), 256, 0, ctx->stream>>>(
        csr->rb_off.p, csr->rb_blocks, tile, mx.p);
  });
  unsigned long long hm = 0;
  d2h(ctx, &hm, mx.p, 1);
  ctx_sync(ctx);
  return (int64_t)hm;
}

void csr_drop_rb(leo2d_csr* csr) {
  csr_drop_rbw(csr);
  csr->rb_xs_built = false;
  csr->rb_xrel.release();
  csr->rb_xs.release();
  csr->rb_built = false;
  csr->rb_blocks = 0;
  csr->rb_slots = 0;
  csr->rb_tile_warps = 0;
  csr->rb_tile_max_bytes = 0;
  for (int64_t& b : csr->rb_tile_bytes_w) b = 0;
  csr->rb_off.release();
  csr->rb_data.release();
  csr->rb_im.release();
}

bool csr_build_rb(leo2d_ctx* ctx, leo2d_csr* csr) {
  LEO_REQUIRE(csr->reordered && csr->prow.p && csr->pcol.p && csr->pval32.p,
              "row blocks are built from the locality-ordered copy");
  csr_drop_rb(csr);
  const int64_t n = csr->n;
  const int64_t nrb = (n + kRbRows - 1) / kRbRows;
  DevBuf<int64_t> cnt((size_t)nrb);
  csr->rb_off.alloc((size_t)nrb + 1 + kRbOffPad);
  LEO_CUDA(cudaMemsetAsync(csr->rb_off.p, 0, ((size_t)nrb + 1 + kRbOffPad) * sizeof(int64_t), ctx->stream));
  DevBuf<int> err(2);
  DevBuf<unsigned long long> ssum(1);
  LEO_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), ctx->stream));
  LEO_CUDA(cudaMemsetAsync(ssum.p, 0, sizeof(unsigned long long), ctx->stream));
  const size_t smem = (size_t)kRbMaxEnt * sizeof(unsigned long long);
  LEO_CUDA(cudaFuncSetAttribute(k_rb_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // a warp per row block; the blocks with more entries than it sorts go to the
  // block-wide kernel (listed in pass 0, the same list in pass 1)
  DevBuf<int64_t> big((size_t)nrb);
  DevBuf<unsigned long long> n_big(1);
  LEO_CUDA(cudaMemsetAsync(n_big.p, 0, sizeof(unsigned long long), ctx->stream));
  const unsigned wgrid =
      (unsigned)std::min<int64_t>((nrb + kRbWarpsPerCta - 1) / kRbWarpsPerCta, (int64_t)ctx->sm_count * 16);
  launch(ctx, "rb_build", [&] {
    k_rb_build_warp<<<wgrid, kRbWarpsPerCta * 32, 0, ctx->stream>>>(n, nrb, csr->prow.p, csr->pcol.p,
                                                                    csr->pval32.p, nullptr, 0, cnt.p, nullptr,
                                                                    nullptr, nullptr, err.p, ssum.p, big.p, n_big.p);
  });
  unsigned long long hb = 0;
  d2h(ctx, &hb, n_big.p, 1);
  ctx_sync(ctx);
  const int64_t nb = (int64_t)hb;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nb, (int64_t)ctx->sm_count * 4));
  if (nb > 0)
    launch(ctx, "rb_build", [&] {
      k_rb_build<<<grid, kRbBuildThreads, smem, ctx->stream>>>(n, nrb, csr->prow.p, csr->pcol.p, csr->pval32.p,
                                                                nullptr, 0, cnt.p, nullptr, nullptr, nullptr, err.p,
                                                                ssum.p, big.p, nb);
    });
  int h[2] = {0, 0};
  unsigned long long hs = 0;
  d2h(ctx, h, err.p, 2);
  d2h(ctx, &hs, ssum.p, 1);
  ctx_sync(ctx);
  if (h[0] != 0) {
    csr_drop_rb(csr);
    return false;
  }
  exclusive_scan_i64(ctx, cnt.p, csr->rb_off.p, nrb);
  int64_t total = 0;
  d2h(ctx, &total, csr->rb_off.p + nrb, 1);
  ctx_sync(ctx);
  // the padding past off[nrb] repeats the total (tile copies read it, never use it)
  std::vector<int64_t> pad(kRbOffPad, total);
  h2d(ctx, csr->rb_off.p + nrb + 1, pad.data(), pad.size());
  csr->rb_data.alloc((size_t)std::max<int64_t>(total, 1) * kRbSlotBytes);
  if (csr->complex_h) {
    LEO_REQUIRE(csr->pval_im32.p, "the ordered copy lacks the imaginary parts");
    csr->rb_im.alloc((size_t)std::max<int64_t>(total, 1) * kRbRows);
    LEO_CUDA(cudaMemsetAsync(csr->rb_im.p, 0, (size_t)std::max<int64_t>(total, 1) * kRbRows * sizeof(float),
                             ctx->stream));
  }
  launch(ctx, "rb_build", [&] {
    k_rb_build_warp<<<wgrid, kRbWarpsPerCta * 32, 0, ctx->stream>>>(
        n, nrb, csr->prow.p, csr->pcol.p, csr->pval32.p, csr->complex_h ? csr->pval_im32.p : nullptr, 1, nullptr,
        csr->rb_off.p, csr->rb_data.p, csr->complex_h ? csr->rb_im.p : nullptr, err.p, ssum.p, big.p, n_big.p);
  });
  if (nb > 0)
    launch(ctx, "rb_build", [&] {
      k_rb_build<<<grid, kRbBuildThreads, smem, ctx->stream>>>(
          n, nrb, csr->prow.p, csr->pcol.p, csr->pval32.p, csr->complex_h ? csr->pval_im32.p : nullptr, 1, nullptr,
          csr->rb_off.p, csr->rb_data.p, csr->complex_h ? csr->rb_im.p : nullptr, err.p, ssum.p, big.p, nb);
  });
  ctx_sync(ctx);
  csr->rb_blocks = nrb;
  csr->rb_slots = total;
  csr->rb_union = (int64_t)hs;
  csr->rb_max_slots = h[1];
  csr->rb_patch = csr->reorder_patch;
  csr->rb_built = true;
  return true;
}

int rb_stages(leo2d_ctx* ctx, leo2d_csr* csr, int warps, bool velocity) {
  if (!csr->rb_built) return 0;
  const int64_t stage = rb_stage_bytes(ctx, csr, warps, velocity);
  const int64_t budget = (int64_t)ctx->smem_optin - 6 * 1024;  // static shared memory of the kernel (4.7 KB)
  const int64_t s = std::min<int64_t>(4, budget / std::max<int64_t>(stage, 1));
  return s >= 2 ? (int)std::min<int64_t>(s, std::max(2, ctx->tile_stages)) : 0;
}

size_t rb_smem_bytes(leo2d_ctx* ctx, leo2d_csr* csr, int warps, bool velocity) {
  return (size_t)rb_stages(ctx, csr, warps, velocity) * (size_t)rb_stage_bytes(ctx, csr, warps, velocity);
}

unsigned rb_grid(leo2d_ctx* ctx, const leo2d_csr* csr, int warps) {
  const int64_t tiles = (csr->rb_blocks + warps - 1) / warps;
  const int64_t chunks = (tiles + ctx->tile_chunk - 1) / std::max(1, ctx->tile_chunk);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->sm_count, chunks));
}

void rb_launch_step(leo2d_ctx* ctx, const leo2d_csr* csr, const StepShape& shape, unsigned grid, size_t smem,
                    const float* tn, float* tp, const float* tprev, int first, float alpha, double* partials,
                    const double* prev_partials, double* prev_dots, float* out2) {
  leo2d_csr* m = const_cast<leo2d_csr*>(csr);
  const bool vel = out2 != nullptr;
  if (vel) LEO_REQUIRE(csr->rb_xs_built && !csr->complex_h, "the velocity step needs the slots' positions");
  RbArgs a{};
  a.n = csr->n;
  a.nrb = csr->rb_blocks;
  a.off = csr->rb_off.p;
  a.data = csr->rb_data.p;
  a.tn = tn;
  a.tp = tp;
  a.tprev = tprev;
  a.first = first;
  a.alpha = alpha;
  a.partials = partials;
  a.prev_partials = prev_partials;
  a.prev_dots = prev_dots;
  const int w = shape.rb_warps;
  a.stages = rb_stages(ctx, m, w, vel);
  LEO_REQUIRE(a.stages >= 2, "row-block tiles too large for shared memory");
  a.chunk = std::max(1, ctx->tile_chunk);
  a.off_bytes = rb_off_bytes(w);
  a.stage_bytes = (int)rb_stage_bytes(ctx, m, w, vel);
  a.im = csr->complex_h ? csr->rb_im.p : nullptr;
  a.panel_at = (int)(a.stage_bytes - rb_panel_bytes(ctx, m, w, vel));
  LEO_REQUIRE((size_t)a.stages * a.stage_bytes <= smem, "row-block shared memory changed since setup");
  a.spin_limit = ctx->spin_limit;
  a.status = ctx->status.p;
  a.never_wait = ctx->test_unsatisfied_wait;
  a.xrel = vel ? csr->rb_xrel.p : nullptr;
  a.xs = vel ? csr->rb_xs.p : nullptr;
  a.out2 = out2;
  auto go = [&](auto kern, int warps) {
    LEO_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    launch(ctx, vel ? "cheb_step_vel" : "cheb_step", [&] { kern<<<grid, warps * 32, smem, ctx->stream>>>(a); });
  };
  if (vel) {
    // the velocity step: T_{n+1} and D T_n from the same gathers
    // (the variants whose two accumulators fit the registers without spills)
    const int vkey = (w / 8) * 100 + (shape.rb_packed ? 10 : 0) + (shape.rb_unroll == 8 ? 1 : 0);
    switch (vkey) {
      case 200: return go(k_cheb_rb<16, false, 4, false, true>, 16);
      case 201: return go(k_cheb_rb<16, false, 8, false, true>, 16);
      case 210: return go(k_cheb_rb<16, true, 4, false, true>, 16);
      case 211: return go(k_cheb_rb<16, true, 8, false, true>, 16);
      case 300: return go(k_cheb_rb<24, false, 4, false, true>, 24);
    }
    fail(LEO2D_ERR_BAD_ARG, "the velocity row-block step runs 16 warps, or 24 with scalar FMAs and 4 batches");
  }
  if (csr->complex_h) {
    switch (w) {
      case 24: return go(k_cheb_rb<24, false, 4, true>, 24);
      case 16: return go(k_cheb_rb<16, false, 4, true>, 16);
      case 8: return go(k_cheb_rb<8, false, 4, true>, 8);
    }
    fail(LEO2D_ERR_BAD_ARG, "the complex row-block step runs 8, 16 or 24 warps");
  }
  // variant: warps (16, 24, 32) x FMA form x slot batches in flight (4, 8)
  const int key = (w / 8) * 100 + (shape.rb_packed ? 10 : 0) + (shape.rb_unroll == 8 ? 1 : 0);
#define LEO2D_RB_CASE(W, P, U) \
  case (W / 8) * 100 + (P ? 10 : 0) + (U == 8 ? 1 : 0): return go(k_cheb_rb<W, P, U>, W);
#define LEO2D_RB_W(W)         \
  LEO2D_RB_CASE(W, false, 4) \
  LEO2D_RB_CASE(W, false, 8) \
  LEO2D_RB_CASE(W, true, 4)  \
  LEO2D_RB_CASE(W, true, 8)
  switch (key) {
    LEO2D_RB_W(16)
    LEO2D_RB_W(24)
    LEO2D_RB_W(32)
  }
#undef LEO2D_RB_W
#undef LEO2D_RB_CASE
  fail(LEO2D_ERR_BAD_ARG, "row-block warps must be 16, 24 or 32 and batches 4 or 8");
}

size_t rb_batch_smem(leo2d_ctx* ctx, const leo2d_csr* const* csrs, int n, int warps) {
  size_t m = 0;
  for (int f = 0; f < n; ++f) {
    leo2d_csr* c = const_cast<leo2d_csr*>(csrs[f]);
    LEO_REQUIRE(rb_stages(ctx, c, warps) >= 2, "row blocks of a batched matrix do not fit shared memory");
    m = std::max(m, rb_smem_bytes(ctx, c, warps));
  }
  return m;
}

int64_t rb_tiles(const leo2d_csr* csr, int warps) { return (csr->rb_blocks + warps - 1) / warps; }

void rb_batch_launch(leo2d_ctx* ctx, const RbBatchFlake* fl, const int* block_first, int nflakes, int warps,
                     size_t smem) {
  LEO_REQUIRE(nflakes >= 1 && nflakes <= kRbBatchMax, "a row-block batch holds 1..64 matrices");
  LEO_REQUIRE(warps == 24, "the batched row-block step runs 24 warps");
  RbBatchParams p;
  std::memset(&p, 0, sizeof(p));
  p.nflakes = nflakes;
  for (int f = 0; f <= nflakes; ++f) p.block_first[f] = block_first[f];
  for (int f = 0; f < nflakes; ++f) {
    leo2d_csr* m = const_cast<leo2d_csr*>(fl[f].csr);
    LEO_REQUIRE(m->rb_built && !m->complex_h, "a batched matrix lacks its row blocks");
    RbArgs& a = p.f[f];
    a.n = m->n;
    a.nrb = m->rb_blocks;
    a.off = m->rb_off.p;
    a.data = m->rb_data.p;
    a.tn = fl[f].tn;
    a.tp = fl[f].tp;
    a.tprev = nullptr;
    a.first = fl[f].first;
    a.alpha = 0.0f;
    a.partials = fl[f].partials;
    a.prev_partials = fl[f].prev_partials;
    a.prev_dots = fl[f].prev_dots;
    a.stages = rb_stages(ctx, m, warps);
    LEO_REQUIRE(a.stages >= 2 && (size_t)a.stages * rb_stage_bytes(ctx, m, warps, false) <= smem,
                "batched row-block shared memory changed since setup");
    a.chunk = std::max(1, ctx->tile_chunk);
    a.off_bytes = rb_off_bytes(warps);
    a.stage_bytes = (int)rb_stage_bytes(ctx, m, warps, false);
    a.panel_at = (int)(a.stage_bytes - rb_panel_bytes(ctx, m, warps, false));
    a.spin_limit = ctx->spin_limit;
    a.status = ctx->status.p;
    a.never_wait = ctx->test_unsatisfied_wait;
  }
  auto kern = k_cheb_rb_batch<24, true, 8>;
  LEO_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  launch(ctx, "cheb_batch_step",
         [&] { kern<<<(unsigned)block_first[nflakes], warps * 32, smem, ctx->stream>>>(p); });
}

}  // namespace leo2d

namespace leo2d {

void csr_build_rb_xs(leo2d_ctx* ctx, leo2d_csr* csr) {
  LEO_REQUIRE(csr->rb_built && csr->reordered && csr->pos.p, "slot positions need the row blocks and the geometry");
  if (csr->rb_xs_built) return;
  csr->rb_xrel.alloc((size_t)csr->rb_blocks * kRbRows);
  csr->rb_xs.alloc((size_t)std::max<int64_t>(csr->rb_slots, 1));
  launch(ctx, "rb_xrel", [&] {
    k_rb_xrel<<<grid_for(csr->rb_blocks * 32, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
        csr->n, csr->rb_blocks, csr->rb_off.p, csr->rb_data.p, csr->pos.p, csr->new2old.p, csr->rb_xrel.p,
        csr->rb_xs.p);
  });
  csr->rb_xs_built = true;
}

}  // namespace leo2d

extern "C" leo2d_status leo2d_csr_rb_info(const leo2d_csr* csr, int64_t* row_blocks, int64_t* slots,
                                          int64_t* union_slots, int32_t* max_slots, int64_t* max_tile_bytes) {
  if (!csr) return LEO2D_ERR_BAD_ARG;
  const bool b = csr->rb_built;
  if (row_blocks) *row_blocks = b ? csr->rb_blocks : 0;
  if (slots) *slots = b ? csr->rb_slots : 0;
  if (union_slots) *union_slots = b ? csr->rb_union : 0;
  if (max_slots) *max_slots = b ? csr->rb_max_slots : 0;
  if (max_tile_bytes) *max_tile_bytes = b ? csr->rb_tile_max_bytes : 0;
  return LEO2D_OK;
}
