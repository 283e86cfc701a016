// step_kernels.cuh - device code of the fused Chebyshev step, shared by the
// single-matrix drivers (kpm.cu, cond.cu through Recursion) and the batched
// multi-flake driver (batch.cu). Included by .cu files only; everything is in
// an anonymous namespace, so each translation unit instantiates its own kernels.
#pragma once

#include <cstring>
#include <type_traits>

#include "kpm.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

template <typename T, int V>
struct VT;
template <> struct VT<float, 1> { using t = float; };
template <> struct VT<float, 2> { using t = float2; };
template <> struct VT<float, 4> { using t = float4; };
template <> struct VT<double, 1> { using t = double; };
template <> struct VT<double, 2> { using t = double2; };

template <typename T, int V>
struct Pack {
  T v[V];
};

template <typename T, int V>
__device__ __forceinline__ Pack<T, V> ld_gather(const T* p) {
  using vt = typename VT<T, V>::t;
  vt x = __ldg(reinterpret_cast<const vt*>(p));
  Pack<T, V> r;
  memcpy(&r, &x, sizeof(r));
  return r;
}

template <typename T, int V>
__device__ __forceinline__ Pack<T, V> ld_plain(const T* p) {
  using vt = typename VT<T, V>::t;
  vt x = *reinterpret_cast<const vt*>(p);
  Pack<T, V> r;
  memcpy(&r, &x, sizeof(r));
  return r;
}

template <typename T, int V>
__device__ __forceinline__ Pack<T, V> ld_stream(const T* p) {
  using vt = typename VT<T, V>::t;
  vt x = __ldcs(reinterpret_cast<const vt*>(p));
  Pack<T, V> r;
  memcpy(&r, &x, sizeof(r));
  return r;
}

template <typename T, int V>
__device__ __forceinline__ void st_plain(T* p, const Pack<T, V>& r) {
  using vt = typename VT<T, V>::t;
  vt x;
  memcpy(&x, &r, sizeof(r));
  *reinterpret_cast<vt*>(p) = x;
}

template <typename T>
struct StepArgs {
  int64_t n;
  const int64_t* __restrict__ rowptr;
  const int32_t* __restrict__ col;
  const T* __restrict__ val;
  const uint2* __restrict__ ent;  // FP32 entries as (column, value bits) pairs
  const T* __restrict__ tn;  // T_n (gathered)
  T* __restrict__ tp;        // T_{n-1} in, T_{n+1} out
  int first;                 // step 0: T_1 = H~ T_0
  T alpha;                   // y = alpha H~ x (- T_{n-1} unless first); 0 means the default 1 / 2
  const T* __restrict__ tprev;  // T_{n-1} when it is not stored at tp (null: read tp)
  int rows_per_item;
  double* __restrict__ partials;             // this step: [grid][C][2]
  const double* __restrict__ prev_partials;  // previous step's partials, or null
  double* __restrict__ prev_dots;            // where the previous step's dots go
};

// Fixed-order tree reduction of partials[b][t] over b < nb into out[t], for the
// values t assigned to this block.
// `bid` / `nblk`: this block's index and the block count of its group (the grid,
// or the blocks of one flake in a batched launch).
template <int C, int NT = kThreads>
__device__ __forceinline__ void reduce_prev(const double* __restrict__ partials,
                                            double* __restrict__ out, int nb, int bid, int nblk) {
  constexpr int kPow = NT >= 512 ? 512 : 256;  // tree over the first kPow lanes
  __shared__ double red[kPow];
  for (int t = bid; t < 2 * C; t += nblk) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += NT) s += __ldcg(partials + (size_t)b * 2 * C + t);
    for (int base = 0; base < NT; base += kPow) {  // fold lanes >= kPow in, in order
      if ((int)threadIdx.x >= base && (int)threadIdx.x < base + kPow) {
        if (base == 0) red[threadIdx.x] = s;
        else red[threadIdx.x - base] += s;
      }
      __syncthreads();
    }
    for (int w = kPow / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[t] = red[0];
    __syncthreads();
  }
}

template <typename T, int V, int LPR>
__global__ void __launch_bounds__(kThreads, 3) k_cheb_step(const StepArgs<T> a) {
  constexpr int C = V * LPR;
  constexpr int RPW = 32 / LPR;
  using Acc = T;  // FP32 recursion accumulates rows in FP32, FP64 mode in FP64
  if (a.prev_partials) reduce_prev<C>(a.prev_partials, a.prev_dots, gridDim.x, blockIdx.x, gridDim.x);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = lane / LPR, sub = lane % LPR;
  const unsigned gmask = LPR == 32 ? 0xffffffffu : (((1u << LPR) - 1u) << (slot * LPR));
  const int64_t item_rows = (int64_t)a.rows_per_item * RPW;
  const int64_t n_items = (a.n + item_rows - 1) / item_rows;
  const int64_t warps_total = (int64_t)gridDim.x * kWarps;
  const T alpha = a.alpha != T(0) ? a.alpha : (a.first ? T(1) : T(2));
  const T* tprev = a.tprev ? a.tprev : a.tp;

  // dots: T within a work item, then T over kDotFlush items, then FP64 (see
  // tile_body)
  constexpr int kDotFlush = std::is_same<T, float>::value ? 16 : 1;
  double d0[V], d1[V];
  T e0[V], e1[V];
  int since_flush = 0;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    d0[v] = d1[v] = 0.0;
    e0[v] = e1[v] = T(0);
  }

  for (int64_t item = (int64_t)blockIdx.x * kWarps + warp; item < n_items; item += warps_total) {
    Acc f0[V], f1[V];
#pragma unroll
    for (int v = 0; v < V; ++v) f0[v] = f1[v] = Acc(0);
    for (int r = 0; r < a.rows_per_item; ++r) {
      const int64_t row = item * item_rows + (int64_t)r * RPW + slot;
      const bool valid = row < a.n;
      const int64_t beg = valid ? a.rowptr[row] : 0;
      const int64_t end = valid ? a.rowptr[row + 1] : 0;
      T acc[V];
#pragma unroll
      for (int v = 0; v < V; ++v) acc[v] = T(0);
      for (int64_t p = beg; p < end; p += LPR) {
        const int cnt = (end - p) < (int64_t)LPR ? (int)(end - p) : LPR;
        int c_mine = 0;
        T v_mine = T(0);
        if (sub < cnt) {
          c_mine = __ldcs(a.col + p + sub);
          v_mine = __ldcs(a.val + p + sub);
        }
        int k = 0;
        for (; k + 4 <= cnt; k += 4) {
          int c[4];
          T w[4];
          Pack<T, V> x[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            c[u] = __shfl_sync(gmask, c_mine, k + u, LPR);
            w[u] = __shfl_sync(gmask, v_mine, k + u, LPR);
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) x[u] = ld_gather<T, V>(a.tn + (int64_t)c[u] * C + sub * V);
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v] += w[u] * x[u].v[v];
        }
        for (; k < cnt; ++k) {
          const int c = __shfl_sync(gmask, c_mine, k, LPR);
          const T w = __shfl_sync(gmask, v_mine, k, LPR);
          const Pack<T, V> x = ld_gather<T, V>(a.tn + (int64_t)c * C + sub * V);
#pragma unroll
          for (int v = 0; v < V; ++v) acc[v] += w * x.v[v];
        }
      }
      if (valid) {
        const int64_t off = row * C + sub * V;
        const Pack<T, V> xn = ld_gather<T, V>(a.tn + off);
        Pack<T, V> y;
        if (a.first) {
#pragma unroll
          for (int v = 0; v < V; ++v) y.v[v] = alpha * acc[v];
        } else {
          const Pack<T, V> xp = ld_plain<T, V>(tprev + off);
#pragma unroll
          for (int v = 0; v < V; ++v) y.v[v] = alpha * acc[v] - xp.v[v];
        }
        st_plain<T, V>(a.tp + off, y);
#pragma unroll
        for (int v = 0; v < V; ++v) {
          f0[v] += xn.v[v] * xn.v[v];
          f1[v] += y.v[v] * xn.v[v];
        }
      }
    }
#pragma unroll
    for (int v = 0; v < V; ++v) {
      e0[v] += f0[v];
      e1[v] += f1[v];
    }
    if (++since_flush == kDotFlush) {  // warp-uniform
      since_flush = 0;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        d0[v] += (double)e0[v];
        d1[v] += (double)e1[v];
        e0[v] = e1[v] = T(0);
      }
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v) {
    d0[v] += (double)e0[v];
    d1[v] += (double)e1[v];
  }

  // combine the row slots of the warp (lanes with equal `sub`)
#pragma unroll
  for (int o = LPR; o < 32; o <<= 1)
#pragma unroll
    for (int v = 0; v < V; ++v) {
      d0[v] += __shfl_xor_sync(0xffffffffu, d0[v], o);
      d1[v] += __shfl_xor_sync(0xffffffffu, d1[v], o);
    }
  __shared__ double wsum[kWarps][2 * C];
  if (slot == 0) {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      wsum[warp][2 * (sub * V + v)] = d0[v];
      wsum[warp][2 * (sub * V + v) + 1] = d1[v];
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 2 * C; t += kThreads) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) s += wsum[w][t];
    a.partials[(size_t)blockIdx.x * 2 * C + t] = s;
  }
}

template <int C>
__global__ void __launch_bounds__(kThreads) k_reduce_partials(const double* __restrict__ partials,
                                                              double* __restrict__ out, int nb) {
  reduce_prev<C>(partials, out, nb, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------- tiled step (bulk copies)
//
// Same step, with the matrix stream decoupled from the gathers: a block takes
// tiles of TR consecutive rows; an elected thread copies each tile's row
// pointers, column indices and values into shared memory with
// cp.async.bulk (completion counted on an mbarrier), double-buffered so the
// copy of tile i+2 runs while tile i is computed. Lanes then read (col, val)
// from shared memory (broadcast within a row slot) and spend their memory
// parallelism on the gathers of T_n only. Ranges are rounded outward to 16-byte
// multiples; the CSR arrays carry kCsrPad elements of padding for this.

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_cta(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Waits for the phase of `bar` with the given parity; gives up after `limit`
// polls or two seconds, whichever comes first, and returns whether it completed.
// A phase already complete costs one poll (the timer is read only after that).
__device__ __forceinline__ bool bounded_wait(uint64_t* bar, uint32_t parity, uint64_t limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint64_t k = 0; k < limit; ++k) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((k & 255) == 255 && global_ns() - t0 > 2000000000ull) return false;
  }
  return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

struct TileLayout {
  int stages;        // shared-memory stages (2..4)
  int chunk;         // consecutive tiles a block takes before jumping by the grid
  int tile_rows;     // TR
  int cap;           // entries per stage (multiple of 4)
  int rp_bytes;      // (TR + 4) * 8 rounded to 128
  int col_bytes;     // cap * 4 rounded to 128
  int stage_bytes;   // rp + col + val, rounded to 128
};

template <typename T>
struct TileArgs {
  StepArgs<T> s;
  TileLayout lay;
  uint64_t spin_limit;
  int* status;
  int never_wait;  // test hook: wait on a barrier that nobody completes
};

// One block's share of a tiled step: `bid` of `nblk` blocks working on the
// matrix of `ta` (the whole grid, or one flake's group of a batched launch).
template <typename T, int V, int LPR, int WARPS>
__device__ __forceinline__ void tile_body(const TileArgs<T>& ta, const int bid, const int nblk) {
  constexpr int C = V * LPR;
  constexpr int RPW = 32 / LPR;
  constexpr int NS = WARPS * RPW;
  constexpr int NT = WARPS * 32;
  // FP32: (column, value) pairs, one 8-byte shared load per entry
  constexpr bool kAoS = std::is_same<T, float>::value;
  constexpr int kMaxStages = 4;
  const StepArgs<T>& a = ta.s;
  const TileLayout& L = ta.lay;
  const int nst = L.stages;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kMaxStages];
  __shared__ int released[kMaxStages];  // warps done with the stage's current tile
  __shared__ int issued[kMaxStages];    // copies issued into the stage so far
  __shared__ __align__(8) uint64_t never;  // test hook barrier: no arrivals
  if (a.prev_partials) reduce_prev<C, NT>(a.prev_partials, a.prev_dots, nblk, bid, nblk);

  const int TR = L.tile_rows;
  const int64_t n_tiles = (a.n + TR - 1) / TR;
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

  // copies of `tile` into `stage` (one lane)
  auto issue = [&](int64_t tile, int stage) {
    const int64_t r0 = tile * TR;
    const int64_t tr = min((int64_t)TR, a.n - r0);
    const int64_t q0 = a.rowptr[r0], q1 = a.rowptr[r0 + tr];
    const int64_t ra = r0 & ~1ll;
    const int64_t rcount = ((r0 + tr + 1 - ra) + 1) & ~1ll;
    const int64_t qa = q0 & ~3ll;
    const int64_t qcount = ((q1 - qa) + 3) & ~3ll;
    unsigned char* st = smem + (size_t)stage * L.stage_bytes;
    issued[stage] += 1;
    if constexpr (kAoS) {
      const uint32_t bytes = (uint32_t)(rcount * 8 + qcount * 8);
      mbar_expect_tx(&full[stage], bytes);
      bulk_g2s(st, a.rowptr + ra, (uint32_t)(rcount * 8), &full[stage]);
      if (qcount > 0) bulk_g2s(st + L.rp_bytes, a.ent + qa, (uint32_t)(qcount * 8), &full[stage]);
    } else {
      const uint32_t bytes = (uint32_t)(rcount * 8 + qcount * (4 + (int64_t)sizeof(T)));
      mbar_expect_tx(&full[stage], bytes);
      bulk_g2s(st, a.rowptr + ra, (uint32_t)(rcount * 8), &full[stage]);
      if (qcount > 0) {
        bulk_g2s(st + L.rp_bytes, a.col + qa, (uint32_t)(qcount * 4), &full[stage]);
        bulk_g2s(st + L.rp_bytes + L.col_bytes, a.val + qa, (uint32_t)(qcount * sizeof(T)), &full[stage]);
      }
    }
  };

  // Runs of `chunk` consecutive tiles are dealt round-robin: consecutive tiles
  // of a block share most of their gathered T_n rows (L1 reuse) while the grid
  // still sweeps the matrix as one band (the rows in flight stay L2-resident).
  const int64_t chunk = L.chunk;
  auto tile_of = [&](int64_t i) -> int64_t {
    return ((int64_t)bid + (i / chunk) * (int64_t)nblk) * chunk + i % chunk;
  };
  if (threadIdx.x == 0)
    for (int i = 0; i < nst; ++i)
      if (tile_of(i) < n_tiles) issue(tile_of(i), i);
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = lane / LPR, sub = lane % LPR;
  const int gslot = warp * RPW + slot;
  const T alpha = a.alpha != T(0) ? a.alpha : (a.first ? T(1) : T(2));
  const T* tprev = a.tprev ? a.tprev : a.tp;
  // dots: T within a tile, then T over kDotFlush tiles, then FP64 (in FP32 mode
  // the FP64 pipe is a small fraction of the FP32 one: converting every tile's
  // partials would bound the kernel)
  constexpr int kDotFlush = std::is_same<T, float>::value ? 16 : 1;
  double d0[V], d1[V];
  T e0[V], e1[V];
  int since_flush = 0;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    d0[v] = d1[v] = 0.0;
    e0[v] = e1[v] = T(0);
  }

  bool gave_up = false;
  if (ta.never_wait && !bounded_wait(&never, 0u, ta.spin_limit)) {
    if (lane == 0) atomicExch(ta.status, leo2d::kStatusTimeout);
    gave_up = true;
  }

  // Warps advance independently: no block barrier per tile. The last warp to
  // release a stage refills it with the tile nst steps ahead.
  int it = 0;
  for (int64_t tile = tile_of(0); !gave_up && tile < n_tiles; tile = tile_of(++it)) {
    const int stage = it % nst;
    const uint32_t parity = (uint32_t)(it / nst) & 1u;
    if (!bounded_wait(&full[stage], parity, ta.spin_limit)) {
      if (lane == 0) atomicExch(ta.status, leo2d::kStatusTimeout);
      break;
    }
    const unsigned char* st = smem + (size_t)stage * L.stage_bytes;
    const int64_t* rp_s = reinterpret_cast<const int64_t*>(st);
    const int32_t* col_s = reinterpret_cast<const int32_t*>(st + L.rp_bytes);
    const T* val_s = reinterpret_cast<const T*>(st + L.rp_bytes + L.col_bytes);
    const uint2* ent_s = reinterpret_cast<const uint2*>(st + L.rp_bytes);
    const int64_t r0 = tile * TR;
    const int tr = (int)min((int64_t)TR, a.n - r0);
    const int64_t ra = r0 & ~1ll;
    const int64_t qa = rp_s[r0 - ra] & ~3ll;
    T f0[V], f1[V];
#pragma unroll
    for (int v = 0; v < V; ++v) f0[v] = f1[v] = T(0);
    for (int lr = gslot; lr < tr; lr += NS) {
      const int64_t row = r0 + lr;
      const int beg = (int)(rp_s[row - ra] - qa), end = (int)(rp_s[row + 1 - ra] - qa);
      const int64_t off = row * C + sub * V;
      // epilogue operands first: their latency overlaps the gathers
      const Pack<T, V> xn = ld_gather<T, V>(a.tn + off);
      Pack<T, V> xp;
      if (!a.first) xp = ld_stream<T, V>(tprev + off);
      T acc[V];
#pragma unroll
      for (int v = 0; v < V; ++v) acc[v] = T(0);
      // (AoS) entries are read two per 16-byte shared load from an even index;
      // the stage holds 8 entries of slack past the last tile's end for this.
      const int k0 = kAoS ? (beg & ~1) : beg;
      for (int k = k0; k < end; k += 8) {
        int c[8];
        T w[8];
        bool in[8];
        Pack<T, V> x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) in[u] = (k + u >= beg) && (k + u < end);
        if constexpr (kAoS) {
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const uint4 e = reinterpret_cast<const uint4*>(ent_s)[(k >> 1) + h];
            c[2 * h] = (int)e.x;
            w[2 * h] = __uint_as_float(e.y);
            c[2 * h + 1] = (int)e.z;
            w[2 * h + 1] = __uint_as_float(e.w);
          }
        } else {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            c[u] = in[u] ? col_s[k + u] : 0;
            w[u] = in[u] ? val_s[k + u] : T(0);
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (in[u]) {
            x[u] = ld_gather<T, V>(a.tn + (int64_t)c[u] * C + sub * V);
          } else {
            w[u] = T(0);
#pragma unroll
            for (int v = 0; v < V; ++v) x[u].v[v] = T(0);
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
          for (int v = 0; v < V; ++v) acc[v] += w[u] * x[u].v[v];
      }
      Pack<T, V> y;
#pragma unroll
      for (int v = 0; v < V; ++v) y.v[v] = a.first ? alpha * acc[v] : alpha * acc[v] - xp.v[v];
      st_plain<T, V>(a.tp + off, y);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        f0[v] += xn.v[v] * xn.v[v];
        f1[v] += y.v[v] * xn.v[v];
      }
    }
#pragma unroll
    for (int v = 0; v < V; ++v) {
      e0[v] += f0[v];
      e1[v] += f1[v];
    }
    if (++since_flush == kDotFlush) {  // warp-uniform
      since_flush = 0;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        d0[v] += (double)e0[v];
        d1[v] += (double)e1[v];
        e0[v] = e1[v] = T(0);
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
  // after a timeout a copy may still be in flight: it must land before exit.
  // Copies finish in microseconds, so this drain is bounded by time only
  // (two seconds), not by the context's poll limit.
  if (threadIdx.x == 0)
    for (int i = 0; i < nst; ++i)
      if (issued[i] > 0) bounded_wait(&full[i], (uint32_t)(issued[i] - 1) & 1u, ~0ull);

#pragma unroll
  for (int v = 0; v < V; ++v) {
    d0[v] += (double)e0[v];
    d1[v] += (double)e1[v];
  }
#pragma unroll
  for (int o = LPR; o < 32; o <<= 1)
#pragma unroll
    for (int v = 0; v < V; ++v) {
      d0[v] += __shfl_xor_sync(0xffffffffu, d0[v], o);
      d1[v] += __shfl_xor_sync(0xffffffffu, d1[v], o);
    }
  // warps add their column sums in warp order (deterministic)
  __shared__ double bsum[2 * C];
  for (int t = threadIdx.x; t < 2 * C; t += NT) bsum[t] = 0.0;
  __syncthreads();
  for (int w = 0; w < WARPS; ++w) {
    if (warp == w && slot == 0) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        bsum[2 * (sub * V + v)] += d0[v];
        bsum[2 * (sub * V + v) + 1] += d1[v];
      }
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < 2 * C; t += NT) a.partials[(size_t)bid * 2 * C + t] = bsum[t];
}

template <typename T, int V, int LPR, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, WARPS == 8 ? 3 : 1) k_cheb_tile(const TileArgs<T> ta) {
  tile_body<T, V, LPR, WARPS>(ta, (int)blockIdx.x, (int)gridDim.x);
}

// Largest entry count over tiles of `tr` consecutive rows.
__global__ void k_tile_max_nnz(const int64_t* __restrict__ rp, int64_t n, int tr,
                               unsigned long long* out) {
  const int64_t tiles = (n + tr - 1) / tr;
  unsigned long long m = 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tiles;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = t * tr, r1 = min(n, r0 + tr);
    const unsigned long long v = (unsigned long long)(rp[r1] - (rp[r0] & ~3ll));
    m = v > m ? v : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, m, o);
    m = y > m ? y : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// ---------------------------------------------------------------- start vectors

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Random-phase columns: complex vector j of the block -> columns 2j (cos), 2j+1 (sin).
// Column c of complex vector `first + c/2` at original row `row`: cos (even c)
// or sin (odd c) of phi = 2 pi u, u the top 24 bits of Philox4x32-10 word 0 at
// counter (row, vector) and key seed.
__device__ __forceinline__ double phase_entry(int64_t row, int c, uint64_t seed, uint64_t first) {
  const uint64_t vv = first + (uint64_t)(c >> 1);
  uint32_t ctr[4] = {(uint32_t)row, (uint32_t)((uint64_t)row >> 32), (uint32_t)vv, (uint32_t)(vv >> 32)};
  philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
  const double u = (double)(ctr[0] >> 8) * (1.0 / 16777216.0);
  const double phi = 6.283185307179586 * u;
  return (c & 1) ? sin(phi) : cos(phi);
}

// One thread per (row, complex vector): one Philox draw and one FP64 sincos for
// both columns (the values of phase_entry's cos and sin).
template <typename T>
__global__ void k_fill_phase(int64_t n, int C, T* __restrict__ x, uint64_t seed, uint64_t first,
                             int n_complex, const int32_t* __restrict__ new2old) {
  const int V = C >> 1;
  const int64_t total = n * V;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / V;
    const int v = (int)(e % V);
    T re = T(0), im = T(0);
    if (v < n_complex) {
      const int64_t row = new2old ? (int64_t)new2old[r] : r;
      const uint64_t vv = first + (uint64_t)v;
      uint32_t ctr[4] = {(uint32_t)row, (uint32_t)((uint64_t)row >> 32), (uint32_t)vv, (uint32_t)(vv >> 32)};
      philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
      const double u = (double)(ctr[0] >> 8) * (1.0 / 16777216.0);
      double s, c;
      sincos(6.283185307179586 * u, &s, &c);
      re = (T)(float)c;
      im = (T)(float)s;
    }
    x[r * C + 2 * v] = re;
    x[r * C + 2 * v + 1] = im;
  }
}

// Gaussian columns (Box-Muller on Philox).
// (pairs: complex H, vector v in columns 2v (real part) and 2v + 1 (zero))
template <typename T>
__global__ void k_fill_gauss(int64_t n, int C, T* __restrict__ x, uint64_t seed, uint64_t first,
                             int n_vec, const int32_t* __restrict__ new2old, int pairs) {
  const int64_t total = n * C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = new2old ? (int64_t)new2old[e / C] : e / C;
    const int cc = (int)(e % C);
    const int c = pairs ? cc >> 1 : cc;
    T out = T(0);
    if (c < n_vec && !(pairs && (cc & 1))) {
      const uint64_t vv = first + (uint64_t)c;
      uint32_t ctr[4] = {(uint32_t)row, (uint32_t)((uint64_t)row >> 32), (uint32_t)vv, (uint32_t)(vv >> 32)};
      philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
      const double u1 = ((double)(ctr[0] >> 8) + 1.0) * (1.0 / 16777216.0);
      const double u2 = (double)(ctr[1] >> 8) * (1.0 / 16777216.0);
      const double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
      out = sizeof(T) == 4 ? (T)(float)z : (T)z;
    }
    x[e] = out;
  }
}

// Host vectors [R][n] (FP64) -> block columns.
template <typename T>
__global__ void k_fill_from(int64_t n, int C, T* __restrict__ x, const double* __restrict__ src,
                            int n_vec, const int32_t* __restrict__ new2old, int pairs) {
  const int64_t total = n * C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = new2old ? (int64_t)new2old[e / C] : e / C;
    const int cc = (int)(e % C);
    const int c = pairs ? cc >> 1 : cc;
    x[e] = (c < n_vec && !(pairs && (cc & 1))) ? (T)src[(int64_t)c * n + row] : T(0);
  }
}

template <typename T>
__global__ void k_fill_unit(int64_t n, int C, T* __restrict__ x, const int64_t* __restrict__ targets,
                            int n_t, const int32_t* __restrict__ new2old, int pairs) {
  const int64_t total = n * C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = new2old ? (int64_t)new2old[e / C] : e / C;
    const int cc = (int)(e % C);
    const int c = pairs ? cc >> 1 : cc;
    x[e] = (c < n_t && !(pairs && (cc & 1)) && targets[c] == row) ? T(1) : T(0);
  }
}

}  // namespace
