// kpm.cu - the fused Chebyshev step: CSR SpMM over a block of vectors with the
// three-term update and the moment dot products in one pass.
//
// Replaces the inner loop of Locality::computeDosTraceKPM / computeDosKPM
// (src/locality.cpp:6195-6234, 5997-6033): SpMatrix::vectorMultiply
// (src/matrix/spmatrix.cpp:346-360), the T_{n+1} = 2 H~ T_n - T_{n-1} loop and the
// dots <T_n|T_n>, <T_{n+1}|T_n> of the moment doubling.
//
// Layout in HBM
//   H~   CSR: rowptr int64[n+1], col int32[nnz], val fp32[nnz] (fp64 in FP64 mode)
//   T    two row-major blocks n x C (C real columns: a complex random-phase
//        vector is two columns, re and im). One row of a block is C*4 bytes
//        contiguous, so a gather of row `col` by the lanes of a group is one
//        coalesced 128..512-byte read.
// Kernel
//   A warp owns 32/LPR row slots; the LPR lanes of a slot own V consecutive
//   columns each (C = LPR*V). Column indices and values of a row are loaded
//   LPR at a time (coalesced, streaming cache hint: the matrix is read once per
//   step and must not evict the vector block from L2), broadcast with shuffles
//   and used to gather T_n rows with 16/8/4-byte vector loads.
//   Epilogue: T_{n+1} = a H~T_n - T_{n-1} is written over T_{n-1} (each row is
//   read and written by its own slot only), and <T_n|T_n>, <T_{n+1}|T_n> are
//   accumulated per column: FP32 within a work item (<= 16 rows), FP64 across
//   items, warps and blocks.
//   The grid is persistent (a multiple of the SM count); work items of
//   `rows_per_item` consecutive row slots are taken in grid-stride order so the
//   rows in flight form one band and their gathered neighbours stay in L2.
//   Block partials of step k are reduced, in fixed order, by the first 2C blocks
//   of step k+1 (deterministic, no extra launch per step).
// One launch per step; whole runs are captured in CUDA graphs by the batched
// driver (batch.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>
#include <string>
#include <tuple>

#include "kpm.cuh"

using namespace leo2d;

#include "step_kernels.cuh"

namespace {

// ---------------------------------------------------------------- dispatch

template <typename T, int V, int LPR>
void launch_step_t(leo2d_ctx* ctx, unsigned grid, const StepArgs<T>& a) {
  launch(ctx, "cheb_step", [&] { k_cheb_step<T, V, LPR><<<grid, kThreads, 0, ctx->stream>>>(a); });
}

// (V, LPR) of the tiled kernel for a block width: 16-byte gathers per lane (FP32
// V=4, FP64 V=2), except 8 FP32 columns (V=2).
template <typename T, int V, int LPR, int WARPS>
void tile_kernel_w(leo2d_ctx* ctx, unsigned grid, size_t smem, const TileArgs<T>* a, int* occ,
                   size_t set_smem) {
  if (occ) {
    LEO_CUDA(cudaFuncSetAttribute(k_cheb_tile<T, V, LPR, WARPS>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)set_smem));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k_cheb_tile<T, V, LPR, WARPS>, WARPS * 32, set_smem);
    return;
  }
  launch(ctx, "cheb_step",
         [&] { k_cheb_tile<T, V, LPR, WARPS><<<grid, WARPS * 32, smem, ctx->stream>>>(*a); });
}

template <typename T, int V, int LPR>
void tile_kernel_t(leo2d_ctx* ctx, unsigned grid, size_t smem, const TileArgs<T>* a, int* occ,
                   size_t set_smem, int warps) {
  if (warps == 24) return tile_kernel_w<T, V, LPR, 24>(ctx, grid, smem, a, occ, set_smem);
  return tile_kernel_w<T, V, LPR, 8>(ctx, grid, smem, a, occ, set_smem);
}

template <typename T>
void tile_dispatch(leo2d_ctx* ctx, int cols, unsigned grid, size_t smem, const TileArgs<T>* a, int* occ,
                   size_t set_smem, int warps);

template <>
void tile_dispatch<float>(leo2d_ctx* ctx, int cols, unsigned grid, size_t smem, const TileArgs<float>* a,
                          int* occ, size_t set_smem, int warps) {
  switch (cols) {
    case 8: return tile_kernel_t<float, 2, 4>(ctx, grid, smem, a, occ, set_smem, warps);
    case 16: return tile_kernel_t<float, 4, 4>(ctx, grid, smem, a, occ, set_smem, warps);
    case 32: return tile_kernel_t<float, 4, 8>(ctx, grid, smem, a, occ, set_smem, warps);
    case 64: return tile_kernel_t<float, 4, 16>(ctx, grid, smem, a, occ, set_smem, warps);
    case 128: return tile_kernel_t<float, 4, 32>(ctx, grid, smem, a, occ, set_smem, warps);
  }
  fail(LEO2D_ERR_BAD_ARG, "FP32 block width must be 8, 16, 32, 64 or 128 columns");
}

template <>
void tile_dispatch<double>(leo2d_ctx* ctx, int cols, unsigned grid, size_t smem, const TileArgs<double>* a,
                           int* occ, size_t set_smem, int warps) {
  switch (cols) {
    case 8: return tile_kernel_t<double, 2, 4>(ctx, grid, smem, a, occ, set_smem, warps);
    case 16: return tile_kernel_t<double, 2, 8>(ctx, grid, smem, a, occ, set_smem, warps);
    case 32: return tile_kernel_t<double, 2, 16>(ctx, grid, smem, a, occ, set_smem, warps);
    case 64: return tile_kernel_t<double, 2, 32>(ctx, grid, smem, a, occ, set_smem, warps);
  }
  fail(LEO2D_ERR_BAD_ARG, "FP64 block width must be 8, 16, 32 or 64 columns");
}

// Row slots of a block (warps x slots per warp) in the tiled kernel.
int tile_slots(int cols, bool fp64, int warps) {
  const int v = fp64 ? 2 : (cols == 8 ? 2 : 4);
  const int lpr = cols / v;
  return warps * (32 / lpr);
}

template <typename T>
void launch_step(leo2d_ctx* ctx, int cols, unsigned grid, const StepArgs<T>& a);

template <>
void launch_step<float>(leo2d_ctx* ctx, int cols, unsigned grid, const StepArgs<float>& a) {
  switch (cols) {
    case 8: return launch_step_t<float, 1, 8>(ctx, grid, a);
    case 16: return launch_step_t<float, 1, 16>(ctx, grid, a);
    case 32: return launch_step_t<float, 1, 32>(ctx, grid, a);
    case 64: return launch_step_t<float, 2, 32>(ctx, grid, a);
    case 128: return launch_step_t<float, 4, 32>(ctx, grid, a);
  }
  fail(LEO2D_ERR_BAD_ARG, "FP32 block width must be 8, 16, 32, 64 or 128 columns");
}

template <>
void launch_step<double>(leo2d_ctx* ctx, int cols, unsigned grid, const StepArgs<double>& a) {
  switch (cols) {
    case 8: return launch_step_t<double, 1, 8>(ctx, grid, a);
    case 16: return launch_step_t<double, 1, 16>(ctx, grid, a);
    case 32: return launch_step_t<double, 1, 32>(ctx, grid, a);
    case 64: return launch_step_t<double, 2, 32>(ctx, grid, a);
  }
  fail(LEO2D_ERR_BAD_ARG, "FP64 block width must be 8, 16, 32 or 64 columns");
}

void launch_reduce(leo2d_ctx* ctx, int cols, const double* partials, double* out, int nb) {
  const unsigned g = (unsigned)std::min(2 * cols, 1024);
  auto go = [&](auto kern) {
    launch(ctx, "reduce_partials", [&] { kern<<<g, kThreads, 0, ctx->stream>>>(partials, out, nb); });
  };
  switch (cols) {
    case 8: return go(k_reduce_partials<8>);
    case 16: return go(k_reduce_partials<16>);
    case 32: return go(k_reduce_partials<32>);
    case 64: return go(k_reduce_partials<64>);
    case 128: return go(k_reduce_partials<128>);
  }
  fail(LEO2D_ERR_BAD_ARG, "unsupported block width");
}

template <typename T, int V, int LPR>
int occupancy_t() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_cheb_step<T, V, LPR>, kThreads, 0);
  return b;
}

int occupancy(int cols, bool fp64) {
  if (!fp64) {
    switch (cols) {
      case 8: return occupancy_t<float, 1, 8>();
      case 16: return occupancy_t<float, 1, 16>();
      case 32: return occupancy_t<float, 1, 32>();
      case 64: return occupancy_t<float, 2, 32>();
      case 128: return occupancy_t<float, 4, 32>();
    }
  } else {
    switch (cols) {
      case 8: return occupancy_t<double, 1, 8>();
      case 16: return occupancy_t<double, 1, 16>();
      case 32: return occupancy_t<double, 1, 32>();
      case 64: return occupancy_t<double, 2, 32>();
    }
  }
  return 1;
}

// out[c] = sum_i x[i][c] y[i][c] in FP64, one block per column, fixed order.
__global__ void __launch_bounds__(256) k_col_dots(int64_t n, int C, const float* __restrict__ x,
                                                  const float* __restrict__ y, double* __restrict__ out) {
  __shared__ double red[256];
  const int c = blockIdx.x;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += (double)x[i * C + c] * (double)y[i * C + c];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = red[0];
}

template <typename T>
void enqueue_steps(Recursion& r) {
  leo2d_ctx* ctx = r.ctx;
  const int C = r.shape.cols;
  for (int k = 0; k < r.steps; ++k) {
    if constexpr (std::is_same<T, float>::value) {
      if (r.direct) {
        const float* tk = reinterpret_cast<const float*>(r.buf(k % 2));
        launch(ctx, "direct_dots", [&] {
          k_col_dots<<<C, 256, 0, ctx->stream>>>(r.n, C, tk, r.start, r.direct + (size_t)k * C);
        });
      }
    }
    StepArgs<T> a;
    a.n = r.n;
    a.ent = r.use_perm ? r.csr->pent.p : r.csr->ent.p;  // (Recursion::step selects dxH itself)
    if (r.use_perm) {
      a.rowptr = r.csr->prow.p;
      a.col = r.csr->pcol.p;
      a.val = r.shape.fp64 ? reinterpret_cast<const T*>(r.csr->pval64.p)
                           : reinterpret_cast<const T*>(r.csr->pval32.p);
    } else {
      a.rowptr = r.csr->rowptr.p;
      a.col = r.csr->col.p;
      a.val = r.shape.fp64 ? reinterpret_cast<const T*>(r.csr->val64.p)
                           : reinterpret_cast<const T*>(r.csr->val32.p);
    }
    a.tn = reinterpret_cast<const T*>(r.buf(k % 2));
    a.tp = reinterpret_cast<T*>(r.buf((k + 1) % 2));
    a.first = k == 0;
    a.alpha = T(0);
    a.tprev = nullptr;
    a.rows_per_item = r.shape.rows_per_item;
    a.partials = r.partials.p + (size_t)(k % 2) * r.grid * 2 * C;
    a.prev_partials = k == 0 ? nullptr : r.partials.p + (size_t)((k + 1) % 2) * r.grid * 2 * C;
    a.prev_dots = k == 0 ? nullptr : r.dots.p + (size_t)(k - 1) * 2 * C;
    if constexpr (std::is_same<T, float>::value) {
      if (r.shape.tc) {
        tc_launch_step(ctx, r.csr, C, r.grid, r.dyn_smem, a.tn, a.tp, nullptr, a.first, 0.0f, a.partials,
                       a.prev_partials, a.prev_dots);
        continue;
      }
      if (r.shape.rt) {
        rt_launch_step(ctx, r.csr, r.shape, r.grid, r.dyn_smem, a.tn, a.tp, nullptr, a.first, 0.0f, a.partials,
                       a.prev_partials, a.prev_dots);
        continue;
      }
      if (r.shape.rb && r.shape.rb_window) {
        rbw_launch_step(ctx, r.csr, r.shape, r.grid, r.dyn_smem, a.tn, a.tp, nullptr, a.first, 0.0f, a.partials,
                        a.prev_partials, a.prev_dots);
        continue;
      }
      if (r.shape.rb) {
        rb_launch_step(ctx, r.csr, r.shape, r.grid, r.dyn_smem, a.tn, a.tp, nullptr, a.first, 0.0f, a.partials,
                       a.prev_partials, a.prev_dots);
        continue;
      }
    }
    if (r.shape.tiled) {
      TileArgs<T> ta{};
      ta.s = a;
      ta.lay = TileLayout{r.tile_stages, r.tile_chunk, r.tile_rows, r.tile_cap, r.tile_rp_bytes, r.tile_col_bytes,
                          r.tile_stage_bytes};
      ta.spin_limit = ctx->spin_limit;
      ta.status = ctx->status.p;
      ta.never_wait = ctx->test_unsatisfied_wait;
      tile_dispatch<T>(ctx, C, r.grid, r.dyn_smem, &ta, nullptr, 0, r.shape.warps);
    } else {
      launch_step<T>(ctx, C, r.grid, a);
    }
  }
  launch_reduce(ctx, C, r.partials.p + (size_t)((r.steps - 1) % 2) * r.grid * 2 * C,
                r.dots.p + (size_t)(r.steps - 1) * 2 * C, (int)r.grid);
}

struct ShapeKey {
  const leo2d_csr* csr;
  int64_t n, nnz;
  bool fp64;
  int cols;
  bool operator<(const ShapeKey& o) const {
    return std::tie(csr, n, nnz, fp64, cols) < std::tie(o.csr, o.n, o.nnz, o.fp64, o.cols);
  }
};
struct Tuned {
  int rows = 0, warps = 0;
  bool tc = false;  // the tensor-core step won for this block width
  bool rb = false;  // the row-block step won for this block width
  int rb_warps = 0, rb_unroll = 0;
  bool rb_packed = true;
  bool rb_window = false;
  bool rt = false;  // the 8-row tensor-core step won for this block width
  int rt_warps = 0, rt_depth = 0;
  int rt_stage = 0;
  int rt_rows = 8;
};
std::map<std::pair<leo2d_ctx*, ShapeKey>, Tuned> g_shape_cache;
// best block width per (context, matrix, precision, columns requested)
std::map<std::pair<leo2d_ctx*, ShapeKey>, int> g_block_cache;

}  // namespace

namespace leo2d {

void Recursion::setup(leo2d_ctx* c, const leo2d_csr* m, StepShape s, int steps_) {
  ctx = c;
  csr = m;
  shape = s;
  n = m->n;
  steps = steps_;
  LEO_REQUIRE(m->nnz == 0 || (s.fp64 ? m->val64.p != nullptr : m->val32.p != nullptr),
              "matrix has no values");
  leo2d_csr* mm = const_cast<leo2d_csr*>(m);
  const bool can_perm = allow_perm && m->pos.p != nullptr && m->nnz > 0;
  if (shape.tc && !can_perm) shape.tc = false;
  if (m->complex_h) {
    LEO_REQUIRE((shape.rb || shape.rt) && can_perm && !s.fp64 && s.cols == 32 && ctx->reorder != 0,
                "a complex Hamiltonian needs a row-block step (FP32, 32 columns, locality ordering on)");
    if (shape.rt) {  // the complex 8-row step's one launch form
      shape.rt_stage = 1;
      shape.rt_rows = 8;
      shape.rt_depth = 3;
      if (shape.rt_warps != 12) shape.rt_warps = 16;
    }
  }
  if (shape.rb && (!can_perm || s.fp64 || s.cols != 32 || ctx->reorder == 0)) shape.rb = false;
  if (shape.rt && (!can_perm || s.fp64 || s.cols != 32 || ctx->reorder == 0)) shape.rt = false;
  if (shape.rt) shape.rb = false;
  if (shape.rb || shape.rt) shape.tc = false;
  const bool want_perm = can_perm && (shape.tc || shape.rb || shape.rt || ctx->reorder == 1 ||
                                      (ctx->reorder == -1 && n >= 100000));
  const double patch = reorder_patch_for(ctx, shape.rb || shape.rt);
  if (want_perm && (!m->reordered || (s.fp64 && !m->reorder_fp64) || m->reorder_patch != patch ||
                    m->reorder_curve_req != ctx->reorder_curve))
    csr_build_reordered(ctx, mm, patch, s.fp64 || m->reorder_fp64, ctx->reorder_curve != 0);
  use_perm = want_perm;
  if (shape.tc) {
    // tensor-core tiles of the locality-ordered copy (built once per matrix)
    if (!m->tc_built || m->tc_patch != m->reorder_patch) csr_build_tc(ctx, mm);
    if (m->tc_built && tc_smem_bytes(m, s.cols) <= ctx->smem_optin) {
      dyn_smem = tc_smem_bytes(m, s.cols);
      grid = (unsigned)std::min<int64_t>((int64_t)ctx->sm_count, m->tc_tiles);
      shape.tiled = false;
    } else {
      shape.tc = false;  // a tile too wide for the tensor-core step: the gather kernels run
    }
  }
  if (shape.rb) {
    // row blocks of the locality-ordered copy (built once per matrix)
    if (!m->rb_built || m->rb_patch != m->reorder_patch) csr_build_rb(ctx, mm);
    // a complex H has no other step kernel: narrower tiles when 24 blocks do not fit
    if (m->complex_h && m->rb_built)
      for (int w : {24, 16, 8})
        if (rb_stages(ctx, mm, w) >= 2) {
          shape.rb_warps = w;
          break;
        }
    if (shape.rb_window && m->rb_built && !m->rbw_built) csr_build_rbw(ctx, mm);
    if (shape.rb_window && !(m->rbw_built && rbw_stages(ctx, mm) >= 2)) shape.rb_window = false;
    if (shape.rb_window) {
      dyn_smem = rbw_smem_bytes(ctx, mm);
      grid = rbw_grid(ctx, m);
      shape.tiled = false;
    } else if (m->rb_built && rb_stages(ctx, mm, shape.rb_warps) >= 2) {
      dyn_smem = rb_smem_bytes(ctx, mm, shape.rb_warps);
      grid = rb_grid(ctx, m, shape.rb_warps);
      shape.tiled = false;
    } else {
      LEO_REQUIRE(!m->complex_h, "row blocks of the complex Hamiltonian do not fit shared memory");
      shape.rb = false;  // blocks too wide for the row-block step: the gather kernels run
    }
  }
  if (shape.rt) {
    // 8-row blocks of the locality-ordered copy, stored for this launch shape
    const int w = shape.rt_warps;
    const int panel = m->complex_h ? 16 : shape.rt_rows;  // complex: real and imaginary panels
    const bool fits = rt_smem_bytes(w, shape.rt_depth, shape.rt_stage, panel) + 8 * 1024 <= ctx->smem_optin;
    if (fits && csr_build_rt(ctx, mm, w, rt_group_of(ctx), rt_chunk_of(ctx), shape.rt_rows)) {
      dyn_smem = rt_smem_bytes(w, shape.rt_depth, shape.rt_stage, panel);
      grid = m->rt_grid;
      shape.tiled = false;
    } else {
      LEO_REQUIRE(!m->complex_h, "the complex 8-row blocks do not build here: step_kernel 3 runs the 4-row step");
      shape.rt = false;  // a block too heavy for the 8-row build: the gather kernels run
    }
  }
  if (shape.tiled && !shape.tc && !shape.rb && !shape.rt) {
    const int ns = tile_slots(s.cols, s.fp64, s.warps);
    const int ri = s.rows_per_item > 0 ? s.rows_per_item : std::max(1, 32 / ns);
    tile_rows = ns * ri;
    int& cached_rows = use_perm ? mm->perm_tile_rows : mm->tile_rows_cached;
    int64_t& cached_max = use_perm ? mm->perm_tile_max_nnz : mm->tile_max_nnz;
    if (cached_rows != tile_rows) {
      DevBuf<unsigned long long> mx(1);
      LEO_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), ctx->stream));
      const int64_t tiles = (n + tile_rows - 1) / tile_rows;
      const int64_t* rp = use_perm ? m->prow.p : m->rowptr.p;
      launch(ctx, "tile_max_nnz", [&] {
        k_tile_max_nnz<<<grid_for(tiles, 256, (int64_t)ctx->sm_count * 8), 256, 0, ctx->stream>>>(
            rp, n, tile_rows, mx.p);
      });
      unsigned long long h = 0;
      d2h(ctx, &h, mx.p, 1);
      ctx_sync(ctx);
      cached_max = (int64_t)h;
      cached_rows = tile_rows;
    }
    auto up = [](int64_t x, int64_t a_) { return (x + a_ - 1) / a_ * a_; };
    tile_cap = (int)up(cached_max + 8, 4);  // + slack for the paired entry reads
    const size_t esz = s.fp64 ? sizeof(double) : sizeof(float);
    tile_rp_bytes = (int)up((int64_t)(tile_rows + 4) * 8, 128);
    if (s.fp64) {
      tile_col_bytes = (int)up((int64_t)tile_cap * 4, 128);
      tile_stage_bytes = (int)up(tile_rp_bytes + tile_col_bytes + (int64_t)tile_cap * esz, 128);
    } else {  // (column, value) pairs
      tile_col_bytes = (int)up((int64_t)tile_cap * 8, 128);
      tile_stage_bytes = (int)up(tile_rp_bytes + tile_col_bytes, 128);
    }
    tile_stages = ctx->tile_stages;
    tile_chunk = ctx->tile_chunk;
    dyn_smem = (size_t)tile_stages * tile_stage_bytes;
    if (dyn_smem + 24 * 1024 > ctx->smem_optin) {
      shape.tiled = false;  // rows too heavy for a staged tile: stream from registers
    } else {
      int occ = 0;
      if (s.fp64) tile_dispatch<double>(ctx, s.cols, 0, 0, nullptr, &occ, dyn_smem, s.warps);
      else tile_dispatch<float>(ctx, s.cols, 0, 0, nullptr, &occ, dyn_smem, s.warps);
      const int64_t tiles = (n + tile_rows - 1) / tile_rows;
      const int64_t chunks = (tiles + tile_chunk - 1) / tile_chunk;
      int64_t g = (int64_t)ctx->sm_count * std::max(occ, 1);
      if (g > chunks) g = std::max<int64_t>(chunks, 1);
      grid = (unsigned)g;
    }
  }
  if (!shape.tiled && !shape.tc && !shape.rb && !shape.rt) {
    if (shape.rows_per_item <= 0) shape.rows_per_item = 4;
    const int occ = std::max(1, occupancy(s.cols, s.fp64));
    const int lpr = s.cols <= 32 ? s.cols : 32;  // lanes per row slot
    const int64_t item_rows = (int64_t)shape.rows_per_item * (32 / lpr);
    const int64_t items = (n + item_rows - 1) / item_rows;
    int64_t g = (int64_t)ctx->sm_count * occ;
    const int64_t need = (items + kWarps - 1) / kWarps;
    if (g > need) g = std::max<int64_t>(need, 1);
    grid = (unsigned)g;
  }
  const size_t esz = s.fp64 ? sizeof(double) : sizeof(float);
  x0.alloc((size_t)n * s.cols * esz);
  x1.alloc((size_t)n * s.cols * esz);
  partials.alloc((size_t)2 * grid * 2 * s.cols);
  dots.alloc((size_t)steps * 2 * s.cols);
}

template <typename T>
void one_step(Recursion& r, const void* in, void* out, const void* prev, bool first, double alpha, int matrix) {
  leo2d_ctx* ctx = r.ctx;
  const int C = r.shape.cols;
  LEO_REQUIRE(!r.use_perm && !r.shape.tc && !r.shape.rb && !r.shape.rt,
              "a recursion over dxH needs the unpermuted matrix");
  StepArgs<T> a;
  a.n = r.n;
  a.rowptr = r.csr->rowptr.p;
  a.col = r.csr->col.p;
  if (matrix == 0) {
    a.val = r.shape.fp64 ? reinterpret_cast<const T*>(r.csr->val64.p) : reinterpret_cast<const T*>(r.csr->val32.p);
    a.ent = r.csr->ent.p;
  } else {
    LEO_REQUIRE(r.csr->dx64.p, "matrix was built without LEO2D_CSR_WITH_DX");
    a.val = r.shape.fp64 ? reinterpret_cast<const T*>(r.csr->dx64.p) : reinterpret_cast<const T*>(r.csr->dx32.p);
    a.ent = r.csr->entd.p;
  }
  a.tn = reinterpret_cast<const T*>(in);
  a.tp = reinterpret_cast<T*>(out);
  a.tprev = reinterpret_cast<const T*>(prev);
  a.first = first ? 1 : 0;
  a.alpha = (T)alpha;
  a.rows_per_item = r.shape.rows_per_item;
  a.partials = r.partials.p;
  a.prev_partials = nullptr;
  a.prev_dots = nullptr;
  if (r.shape.tiled) {
    TileArgs<T> ta{};
    ta.s = a;
    ta.lay = TileLayout{r.tile_stages, r.tile_chunk, r.tile_rows, r.tile_cap, r.tile_rp_bytes, r.tile_col_bytes,
                        r.tile_stage_bytes};
    ta.spin_limit = ctx->spin_limit;
    ta.status = ctx->status.p;
    ta.never_wait = ctx->test_unsatisfied_wait;
    tile_dispatch<T>(ctx, C, r.grid, r.dyn_smem, &ta, nullptr, 0, r.shape.warps);
  } else {
    launch_step<T>(ctx, C, r.grid, a);
  }
}

void Recursion::step(const void* in, void* out, const void* prev, bool first, double alpha, int matrix) {
  if (shape.fp64) one_step<double>(*this, in, out, prev, first, alpha, matrix);
  else one_step<float>(*this, in, out, prev, first, alpha, matrix);
}

void Recursion::run() {
  if (shape.fp64) enqueue_steps<double>(*this);
  else enqueue_steps<float>(*this);
  if (shape.tiled || shape.tc || shape.rb || shape.rt) ctx_check_status(ctx, "Chebyshev recursion");
}

Recursion::~Recursion() {
  if (graph) cudaGraphExecDestroy(graph);
}

StepShape choose_shape(leo2d_ctx* ctx, const leo2d_csr* csr, bool fp64, int cols_needed,
                       int requested_cols, int requested_rows) {
  StepShape s;
  s.fp64 = fp64;
  if (requested_cols > 0) {
    s.cols = requested_cols;
  } else {
    auto bt = g_block_cache.find({ctx, ShapeKey{csr, csr->n, csr->nnz, fp64, cols_needed}});
    if (bt != g_block_cache.end()) {
      s.cols = bt->second;
    } else {
      // smallest supported width that holds the request, capped at the widest
      const int maxc = fp64 ? 64 : 128;
      int c = 8;
      while (c < cols_needed && c < maxc) c <<= 1;
      s.cols = c;
    }
  }
  if (csr->complex_h) {
    // a complex H runs on the row-block steps only: 16 complex vectors (32
    // columns), FP32, also when fewer columns are needed (a few LDOS targets)
    LEO_REQUIRE(!fp64, "a complex Hamiltonian (magnetic field) runs in FP32");
    LEO_REQUIRE(s.cols == 32 || requested_cols <= 0, "a complex Hamiltonian takes 32-column blocks");
    s.cols = 32;
  }
  auto it = g_shape_cache.find({ctx, ShapeKey{csr, csr->n, csr->nnz, fp64, s.cols}});
  s.rows_per_item = requested_rows > 0 ? requested_rows : (it != g_shape_cache.end() ? it->second.rows : 0);
  if (ctx->tile_warps > 0) s.warps = ctx->tile_warps;
  else if (it != g_shape_cache.end() && it->second.warps > 0) s.warps = it->second.warps;
  else s.warps = (!fp64 && (s.cols == 32 || s.cols == 64)) ? 24 : 8;
  s.tiled = ctx->kernel_variant != 1;
  const bool tc_ok = !fp64 && (s.cols == 32 || s.cols == 64);
  s.tc = tc_ok && (ctx->kernel_variant == 2 ||
                   (ctx->kernel_variant == -1 && it != g_shape_cache.end() && it->second.tc));
  // the row-block step: when asked for, when the autotuner chose it, and by
  // default where the matrix is large enough to be locality-ordered
  const bool rb_ok = !fp64 && s.cols == 32 && ctx->reorder != 0 && csr->pos.p != nullptr && csr->nnz > 0;
  const bool cached = it != g_shape_cache.end();
  if (ctx->kernel_variant == 3) s.rb = rb_ok;
  else if (ctx->kernel_variant == -1) s.rb = rb_ok && (cached ? it->second.rb : (ctx->reorder == 1 || csr->n >= 100000));
  const bool rt_ok = rb_ok;
  if (ctx->kernel_variant == 5) s.rt = rt_ok;
  else if (ctx->kernel_variant == -1) s.rt = rt_ok && (cached ? it->second.rt : s.rb);
  if (s.rt) s.rb = false;
  if (s.rb || s.rt) s.tc = false;
  if (csr->complex_h) {
    s.rb = !s.rt;  // the 4-row step, or the 8-row step when asked for
    s.tc = false;
    s.tiled = true;
  }
  s.rb_warps = ctx->rb_warps > 0 ? ctx->rb_warps : (cached && it->second.rb_warps > 0 ? it->second.rb_warps : 24);
  s.rb_unroll = ctx->rb_unroll > 0 ? ctx->rb_unroll : (cached && it->second.rb_unroll > 0 ? it->second.rb_unroll : 8);
  s.rb_packed = ctx->rb_packed >= 0 ? ctx->rb_packed != 0 : (cached ? it->second.rb_packed : true);
  s.rb_window = ctx->rb_window >= 0 ? ctx->rb_window != 0 : (cached ? it->second.rb_window : false);
  if (csr->complex_h) {
    s.rb_window = false;
    s.rb_warps = 24;
  }
  s.rt_warps = ctx->rt_warps > 0 ? ctx->rt_warps : (cached && it->second.rt_warps > 0 ? it->second.rt_warps : 16);
  s.rt_stage = ctx->rt_stage >= 0 ? ctx->rt_stage : (cached && it->second.rt ? it->second.rt_stage : 1);
  s.rt_depth = ctx->rt_depth > 0 ? ctx->rt_depth : (cached && it->second.rt_depth > 0 ? it->second.rt_depth : 3);
  s.rt_rows = ctx->rt_rows > 0 ? ctx->rt_rows : (cached && it->second.rt ? it->second.rt_rows : 8);
  LEO_REQUIRE(s.rows_per_item >= 0 && s.rows_per_item <= 64, "rows_per_warp must be 0..64");
  return s;
}

void fill_phase(leo2d_ctx* ctx, Recursion& r, uint64_t seed, uint64_t first, int n_complex) {
  const int64_t total = r.n * r.shape.cols;
  const unsigned g = grid_for(total, 256, (int64_t)ctx->sm_count * 32);
  if (r.shape.fp64)
    launch(ctx, "fill_phase", [&] {
      k_fill_phase<double><<<g, 256, 0, ctx->stream>>>(r.n, r.shape.cols, (double*)r.x0.p, seed, first, n_complex, r.perm());
    });
  else
    launch(ctx, "fill_phase", [&] {
      k_fill_phase<float><<<g, 256, 0, ctx->stream>>>(r.n, r.shape.cols, (float*)r.x0.p, seed, first, n_complex, r.perm());
    });
}

void fill_gaussian(leo2d_ctx* ctx, Recursion& r, uint64_t seed, uint64_t first, int n_vec) {
  const int64_t total = r.n * r.shape.cols;
  const unsigned g = grid_for(total, 256, (int64_t)ctx->sm_count * 32);
  if (r.shape.fp64)
    launch(ctx, "fill_gauss", [&] {
      k_fill_gauss<double><<<g, 256, 0, ctx->stream>>>(r.n, r.shape.cols, (double*)r.x0.p, seed, first, n_vec, r.perm(), r.pairs());
    });
  else
    launch(ctx, "fill_gauss", [&] {
      k_fill_gauss<float><<<g, 256, 0, ctx->stream>>>(r.n, r.shape.cols, (float*)r.x0.p, seed, first, n_vec, r.perm(), r.pairs());
    });
}

void fill_host(leo2d_ctx* ctx, Recursion& r, const double* host_vectors, int first_vec, int n_vec) {
  DevBuf<double> src((size_t)n_vec * r.n);
  h2d(ctx, src.p, host_vectors + (size_t)first_vec * r.n, (size_t)n_vec * r.n);
  const int64_t total = r.n * r.shape.cols;
  const unsigned g = grid_for(total, 256, (int64_t)ctx->sm_count * 32);
  if (r.shape.fp64)
    launch(ctx, "fill_host", [&] {
      k_fill_from<double><<<g, 256, 0, ctx->stream>>>(r.n, r.shape.cols, (double*)r.x0.p, src.p, n_vec, r.perm(), r.pairs());
    });
  else
    launch(ctx, "fill_host", [&] {
      k_fill_from<float><<<g, 256, 0, ctx->stream>>>(r.n, r.shape.cols, (float*)r.x0.p, src.p, n_vec, r.perm(), r.pairs());
    });
  LEO_CUDA(cudaStreamSynchronize(ctx->stream));
}

void fill_unit(leo2d_ctx* ctx, Recursion& r, const int64_t* targets, int n_t) {
  DevBuf<int64_t> t(std::max(n_t, 1));
  h2d(ctx, t.p, targets, n_t);
  const int64_t total = r.n * r.shape.cols;
  const unsigned g = grid_for(total, 256, (int64_t)ctx->sm_count * 32);
  if (r.shape.fp64)
    launch(ctx, "fill_unit", [&] {
      k_fill_unit<double><<<g, 256, 0, ctx->stream>>>(r.n, r.shape.cols, (double*)r.x0.p, t.p, n_t, r.perm(), r.pairs());
    });
  else
    launch(ctx, "fill_unit", [&] {
      k_fill_unit<float><<<g, 256, 0, ctx->stream>>>(r.n, r.shape.cols, (float*)r.x0.p, t.p, n_t, r.perm(), r.pairs());
    });
  LEO_CUDA(cudaStreamSynchronize(ctx->stream));
}

// The moments of a non-Hermitian H~ in the reference's order (the complex
// branches of computeDosKPM and computeDosTraceKPM, locality.cpp:6074-6120,
// 6276-6330): mu_j = Re sum_i T_j[i] v[i]
// directly for j < P/2 (complex pairs: re*re - im*im), then for j >= P/4
// mu_2j = 2 <T_j|T_j> - mu_0 and mu_2j+1 = 2 Re <T_j+1|T_j> - mu_1.
void direct_to_moments(const std::vector<double>& direct, const std::vector<double>& dots, int cols, int steps,
                       int n_vec, double* mu_out, int P) {
  for (int v = 0; v < n_vec; ++v) {
    double* mu = mu_out + (size_t)v * P;
    const int cr = 2 * v, ci = 2 * v + 1;
    for (int k = 0; k < steps; ++k) mu[k] = direct[(size_t)k * cols + cr] - direct[(size_t)k * cols + ci];
    for (int k = P / 4; k < steps; ++k) {
      const double D0 = dots[((size_t)k * cols + cr) * 2] + dots[((size_t)k * cols + ci) * 2];
      const double D1 = dots[((size_t)k * cols + cr) * 2 + 1] + dots[((size_t)k * cols + ci) * 2 + 1];
      mu[2 * k] = 2 * D0 - mu[0];
      mu[2 * k + 1] = 2 * D1 - mu[1];
    }
  }
}

void dots_to_moments(const std::vector<double>& dots, int cols, int steps, int group, int n_vec,
                     double* mu_out, int P) {
  for (int v = 0; v < n_vec; ++v) {
    double* mu = mu_out + (size_t)v * P;
    for (int k = 0; k < steps; ++k) {
      double D0 = 0, D1 = 0;
      for (int gidx = 0; gidx < group; ++gidx) {
        const int c = v * group + gidx;
        D0 += dots[((size_t)k * cols + c) * 2];
        D1 += dots[((size_t)k * cols + c) * 2 + 1];
      }
      if (k == 0) {
        mu[0] = D0;
        mu[1] = D1;
      } else {
        mu[2 * k] = 2 * D0 - mu[0];
        mu[2 * k + 1] = 2 * D1 - mu[1];
      }
    }
  }
}

}  // namespace leo2d

// ---------------------------------------------------------------- C ABI

namespace {

void validate_cfg(const leo2d_kpm_cfg* cfg) {
  LEO_REQUIRE(cfg, "cfg is NULL");
  LEO_REQUIRE(cfg->poly_order >= 4 && cfg->poly_order % 4 == 0,
              "poly_order must be a positive multiple of 4 (main.cpp:914-917)");
  LEO_REQUIRE(cfg->precision == LEO2D_FP32 || cfg->precision == LEO2D_FP64, "unknown precision");
  LEO_REQUIRE(cfg->block >= 0 && cfg->rows_per_warp >= 0, "block and rows_per_warp must be >= 0");
}

// For a non-Hermitian H~ (a field on a periodic supercell): keeps a copy of
// each block's start vectors and has the recursion record the direct dots.
struct DirectMoments {
  leo2d_ctx* ctx;
  Recursion& r;
  DevBuf<float> start;
  DevBuf<double> direct;
  DirectMoments(leo2d_ctx* c, const leo2d_csr* csr, Recursion& rr) : ctx(c), r(rr) {
    if (!csr->nonhermitian) return;
    LEO_REQUIRE(!r.shape.fp64, "a complex Hamiltonian runs in FP32");
    start.alloc((size_t)r.n * r.shape.cols);
    direct.alloc((size_t)r.steps * r.shape.cols);
    r.start = start.p;
    r.direct = direct.p;
  }
  bool on() const { return start.p != nullptr; }
  void keep_start() {
    if (on())
      LEO_CUDA(cudaMemcpyAsync(start.p, r.x0.p, (size_t)r.n * r.shape.cols * sizeof(float),
                               cudaMemcpyDeviceToDevice, ctx->stream));
  }
  void moments(const std::vector<double>& dots, int nv, double* mu, int P) {
    std::vector<double> d((size_t)r.steps * r.shape.cols);
    d2h(ctx, d.data(), direct.p, d.size());
    ctx_sync(ctx);
    direct_to_moments(d, dots, r.shape.cols, r.steps, nv, mu, P);
  }
};

// Runs the recursion over the vector blocks of a trace estimate and writes moments.
void run_trace(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg, const double* host_vectors,
               double* mu_out) {
  const int P = cfg->poly_order;
  const int steps = P / 2;
  const bool fp64 = cfg->precision == LEO2D_FP64;
  // complex H: every vector is a (real, imaginary) column pair
  const int group = (cfg->vector_kind == LEO2D_VEC_PHASE || csr->complex_h) ? 2 : 1;
  const int total_cols = cfg->num_vectors * group;
  StepShape shape = choose_shape(ctx, csr, fp64, total_cols, cfg->block, cfg->rows_per_warp);
  LEO_REQUIRE(shape.cols % group == 0, "block width must hold whole complex vectors");
  const int vec_per_block = shape.cols / group;
  Recursion r;
  r.setup(ctx, csr, shape, steps);
  std::vector<double> dots((size_t)steps * 2 * shape.cols);
  DirectMoments dm(ctx, csr, r);
  for (int v0 = 0; v0 < cfg->num_vectors; v0 += vec_per_block) {
    const int nv = std::min(vec_per_block, cfg->num_vectors - v0);
    switch (cfg->vector_kind) {
      case LEO2D_VEC_PHASE: fill_phase(ctx, r, cfg->seed, cfg->first_vector + v0, nv); break;
      case LEO2D_VEC_GAUSSIAN: fill_gaussian(ctx, r, cfg->seed, cfg->first_vector + v0, nv); break;
      case LEO2D_VEC_HOST: fill_host(ctx, r, host_vectors, v0, nv); break;
      default: fail(LEO2D_ERR_BAD_ARG, "unknown vector_kind");
    }
    dm.keep_start();
    r.run();
    d2h(ctx, dots.data(), r.dots.p, dots.size());
    ctx_sync(ctx);
    if (dm.on()) dm.moments(dots, nv, mu_out + (size_t)v0 * P, P);
    else dots_to_moments(dots, shape.cols, steps, group, nv, mu_out + (size_t)v0 * P, P);
  }
  for (size_t i = 0; i < (size_t)cfg->num_vectors * P; ++i)
    if (!std::isfinite(mu_out[i])) fail(LEO2D_ERR_NONFINITE, "non-finite moment (check the spectral bounds)");
}

}  // namespace

extern "C" {

leo2d_status leo2d_kpm_dos(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                           const double* host_vectors, double* mu_out) {
  if (!ctx || !csr || !mu_out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    validate_cfg(cfg);
    LEO_REQUIRE(cfg->num_vectors >= 1, "num_vectors must be >= 1");
    LEO_REQUIRE(cfg->vector_kind != LEO2D_VEC_HOST || host_vectors,
                "LEO2D_VEC_HOST needs host_vectors");
    LEO_CUDA(cudaSetDevice(ctx->device));
    run_trace(ctx, csr, cfg, host_vectors, mu_out);
  });
}

leo2d_status leo2d_kpm_ldos(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                            const int64_t* targets, int64_t num_targets, double* mu_out) {
  if (!ctx || !csr || !mu_out || (num_targets > 0 && !targets)) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    validate_cfg(cfg);
    for (int64_t t = 0; t < num_targets; ++t)
      LEO_REQUIRE(targets[t] >= 0 && targets[t] < csr->n, "target index out of range");
    LEO_CUDA(cudaSetDevice(ctx->device));
    const int P = cfg->poly_order, steps = P / 2;
    const bool fp64 = cfg->precision == LEO2D_FP64;
    const int group = csr->complex_h ? 2 : 1;  // complex H: a (real, imaginary) column pair per target
    StepShape shape = choose_shape(ctx, csr, fp64, (int)std::min<int64_t>(num_targets * group, 128),
                                   cfg->block, cfg->rows_per_warp);
    Recursion r;
    r.setup(ctx, csr, shape, steps);
    std::vector<double> dots((size_t)steps * 2 * shape.cols);
    DirectMoments dm(ctx, csr, r);
    const int per_block = shape.cols / group;
    for (int64_t t0 = 0; t0 < num_targets; t0 += per_block) {
      const int nt = (int)std::min<int64_t>(per_block, num_targets - t0);
      fill_unit(ctx, r, targets + t0, nt);
      dm.keep_start();
      r.run();
      d2h(ctx, dots.data(), r.dots.p, dots.size());
      ctx_sync(ctx);
      if (dm.on()) dm.moments(dots, nt, mu_out + (size_t)t0 * P, P);
      else dots_to_moments(dots, shape.cols, steps, group, nt, mu_out + (size_t)t0 * P, P);
    }
  });
}

}  // extern "C"

// ---------------------------------------------------------------- autotuner

extern "C" leo2d_status leo2d_kpm_autotune(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                                           int32_t* block_out, int32_t* rows_out) {
  if (!ctx || !csr || !cfg) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    validate_cfg(cfg);
    LEO_REQUIRE(cfg->num_vectors >= 1, "num_vectors must be >= 1");
    LEO_CUDA(cudaSetDevice(ctx->device));
    const bool fp64 = cfg->precision == LEO2D_FP64;
    if (csr->complex_h) {  // one step kernel and width for a complex Hamiltonian
      if (block_out) *block_out = 32;
      if (rows_out) *rows_out = 0;
      return;
    }
    const int group = cfg->vector_kind == LEO2D_VEC_PHASE ? 2 : 1;
    const int total_cols = cfg->num_vectors * group;
    const int steps = 8;
    const bool was_profiling = ctx->profiling;
    if (!was_profiling) { ctx_sync(ctx); ctx->profiling = true; }
    double best_cost = INFINITY;
    int best_cols = 0, best_rows = 0;
    const int maxc = fp64 ? 64 : 128;
    for (int cols = 8; cols <= maxc; cols <<= 1) {
      if (cols % group) continue;
      const int passes = (total_cols + cols - 1) / cols;
      double best_c = INFINITY;
      Tuned best_t;
      for (int warps : {8, 24}) {
        if (ctx->tile_warps > 0 && warps != ctx->tile_warps) continue;
        for (int rows : {0, 2}) {
          StepShape sh = choose_shape(ctx, csr, fp64, cols, cols, rows > 0 ? rows : 0);
          sh.rows_per_item = rows;
          sh.warps = warps;
          sh.tc = false;
          sh.rb = false;
          sh.rt = false;
          Recursion r;
          r.setup(ctx, csr, sh, steps);
          fill_phase(ctx, r, 1, 0, cols / 2);
          r.run();  // warm
          ctx_sync(ctx);
          const auto before = ctx->stats["cheb_step"];
          r.run();
          ctx_sync(ctx);
          const auto after = ctx->stats["cheb_step"];
          const double per = (after.ms - before.ms) / std::max<int64_t>(1, after.launches - before.launches);
          if (per < best_c) {
            best_c = per;
            best_t.rows = rows;
            best_t.warps = warps;
          }
        }
      }
      // the windowed tensor-core step (one shape), timed only when asked for: it
      // lost to the gather kernels by 3x on twisted-bilayer flakes and its build
      // took a second per 10M-orbital matrix
      if (!fp64 && (cols == 32 || cols == 64) && ctx->kernel_variant == 2) {
        StepShape sh = choose_shape(ctx, csr, fp64, cols, cols, 0);
        sh.tc = true;
        sh.rb = false;
        sh.rt = false;
        Recursion r;
        r.setup(ctx, csr, sh, steps);
        if (r.shape.tc) {
          fill_phase(ctx, r, 1, 0, cols / 2);
          r.run();  // warm
          ctx_sync(ctx);
          const auto before = ctx->stats["cheb_step"];
          r.run();
          ctx_sync(ctx);
          const auto after = ctx->stats["cheb_step"];
          const double per = (after.ms - before.ms) / std::max<int64_t>(1, after.launches - before.launches);
          if (per < best_c) {
            best_c = per;
            best_t.tc = true;
          }
        }
      }
      // the row-block step where it applies: a few block shapes
      if (!fp64 && cols == 32 && ctx->kernel_variant != 0 && ctx->kernel_variant != 1 &&
          ctx->kernel_variant != 2 && ctx->reorder != 0) {
        struct RbTry { int warps, unroll; bool packed, window; };
        // (the windowed form is timed only when asked for: it measured slower on
        // twisted-bilayer flakes and builds a second copy of the blocks)
        for (const RbTry t : {RbTry{24, 8, true, false}, RbTry{32, 4, true, false}, RbTry{24, 8, false, false},
                              RbTry{16, 8, true, false}, RbTry{16, 4, true, true}}) {
          if ((ctx->rb_window == 1) != t.window) continue;
          StepShape sh = choose_shape(ctx, csr, fp64, cols, cols, 0);
          sh.tc = false;
          sh.rb = true;
          sh.rt = false;
          sh.rb_warps = ctx->rb_warps > 0 ? ctx->rb_warps : t.warps;
          sh.rb_unroll = ctx->rb_unroll > 0 ? ctx->rb_unroll : t.unroll;
          sh.rb_packed = ctx->rb_packed >= 0 ? ctx->rb_packed != 0 : t.packed;
          sh.rb_window = t.window;
          Recursion r;
          r.setup(ctx, csr, sh, steps);
          if (!r.shape.rb) break;
          if (r.shape.rb_window != t.window) continue;
          fill_phase(ctx, r, 1, 0, cols / 2);
          r.run();  // warm
          ctx_sync(ctx);
          const auto before = ctx->stats["cheb_step"];
          r.run();
          ctx_sync(ctx);
          const auto after = ctx->stats["cheb_step"];
          const double per = (after.ms - before.ms) / std::max<int64_t>(1, after.launches - before.launches);
          if (per < best_c) {
            best_c = per;
            best_t.tc = false;
            best_t.rb = true;
            best_t.rb_warps = sh.rb_warps;
            best_t.rb_unroll = sh.rb_unroll;
            best_t.rb_packed = sh.rb_packed;
            best_t.rb_window = sh.rb_window;
          }
        }
      }
      // the 8-row tensor-core step where it applies: a few (warps, depth) shapes
      if (!fp64 && cols == 32 && !csr->complex_h && ctx->reorder != 0 &&
          (ctx->kernel_variant == -1 || ctx->kernel_variant == 5)) {
        struct RtTry { int warps, depth, stage, rows; };
        // (the TMA form, stage 2, is timed only when asked for: 1.8x slower)
        // (16-row blocks: a third fewer k-steps on the 0.5 deg flakes but 1.7x the
        // cost per k-step, 0.69 against 0.60 ms at 2.4M orbitals; kept as a
        // candidate for denser matrices)
        for (const RtTry t : {RtTry{16, 3, 1, 8}, RtTry{20, 3, 1, 8}, RtTry{12, 3, 1, 16}, RtTry{16, 2, 0, 8},
                              RtTry{16, 3, 2, 8}, RtTry{12, 7, 2, 8}}) {
          if (t.stage == 2 && ctx->rt_stage != 2) continue;
          if (ctx->rt_stage >= 0 && ctx->rt_stage != t.stage) continue;
          if (ctx->rt_rows > 0 && ctx->rt_rows != t.rows) continue;
          StepShape sh = choose_shape(ctx, csr, fp64, cols, cols, 0);
          sh.tc = false;
          sh.rb = false;
          sh.rt = true;
          sh.rt_stage = t.stage;
          sh.rt_rows = t.rows;
          sh.rt_warps = ctx->rt_warps > 0 ? ctx->rt_warps : t.warps;
          sh.rt_depth = ctx->rt_depth > 0 ? ctx->rt_depth : t.depth;
          // 16-row blocks come in two launch shapes
          if (t.rows == 16 && !(sh.rt_depth == 3 && (sh.rt_warps == 12 || sh.rt_warps == 16))) continue;
          Recursion r;
          r.setup(ctx, csr, sh, steps);
          if (!r.shape.rt) break;
          fill_phase(ctx, r, 1, 0, cols / 2);
          r.run();  // warm
          ctx_sync(ctx);
          const auto before = ctx->stats["cheb_step"];
          r.run();
          ctx_sync(ctx);
          const auto after = ctx->stats["cheb_step"];
          const double per = (after.ms - before.ms) / std::max<int64_t>(1, after.launches - before.launches);
          if (per < best_c) {
            best_c = per;
            best_t.tc = false;
            best_t.rb = false;
            best_t.rt = true;
            best_t.rt_warps = sh.rt_warps;
            best_t.rt_depth = sh.rt_depth;
            best_t.rt_stage = sh.rt_stage;
            best_t.rt_rows = sh.rt_rows;
          }
          if (ctx->rt_warps > 0 && ctx->rt_depth > 0) break;  // one shape asked for
        }
      }
      g_shape_cache[{ctx, ShapeKey{csr, csr->n, csr->nnz, fp64, cols}}] = best_t;
      const double cost = passes * best_c;
      if (cost < best_cost) {
        best_cost = cost;
        best_cols = cols;
        best_rows = best_t.rows;
      }
    }
    if (!was_profiling) { ctx_sync(ctx); ctx->profiling = false; }
    g_block_cache[{ctx, ShapeKey{csr, csr->n, csr->nnz, fp64, total_cols}}] = best_cols;
    if (block_out) *block_out = best_cols;
    if (rows_out) *rows_out = best_rows;
  });
}

extern "C" leo2d_status leo2d_kpm_step_kernel(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                                              int32_t* kernel, int32_t* block) {
  if (!ctx || !csr || !cfg || !kernel || !block) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    validate_cfg(cfg);
    const bool fp64 = cfg->precision == LEO2D_FP64;
    const int group = cfg->vector_kind == LEO2D_VEC_PHASE ? 2 : 1;
    StepShape s = choose_shape(ctx, csr, fp64, std::max(1, cfg->num_vectors) * group, cfg->block, cfg->rows_per_warp);
    // the demotions Recursion::setup applies before any build
    const bool can_perm = csr->pos.p != nullptr && csr->nnz > 0;
    if (s.rb && (!can_perm || s.fp64 || s.cols != 32 || ctx->reorder == 0)) s.rb = false;
    if (s.rt && (!can_perm || s.fp64 || s.cols != 32 || ctx->reorder == 0)) s.rt = false;
    if (s.tc && !can_perm) s.tc = false;
    *kernel = s.rt ? 5 : s.rb ? (s.rb_window ? 4 : 3) : s.tc ? 2 : s.tiled ? 0 : 1;
    *block = s.cols;
  });
}

// ---------------------------------------------------------------- allocation-free entry point
//
// leo2d_kpm_dos_noalloc: the trace recursion of leo2d_kpm_dos for callers that
// cannot allocate device memory. Its working set (the two vector blocks, the
// block partials and the per-step dots) lives in one file-scope device array.

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;  // 32 MiB, held by every device that loads the library
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch per device (a host-side use of the symbol
// itself would name host memory, not the device array).
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};

__global__ void k_dots_to_moments(const double* __restrict__ dots, int cols, int steps, int n_vec,
                                  double* __restrict__ mu_out, int P) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_vec) return;
  double* mu = mu_out + (size_t)v * P;
  double mu0 = 0.0, mu1 = 0.0;
  for (int k = 0; k < steps; ++k) {
    const double* d = dots + (size_t)k * cols * 2;
    const double D0 = d[2 * (2 * v)] + d[2 * (2 * v + 1)];
    const double D1 = d[2 * (2 * v) + 1] + d[2 * (2 * v + 1) + 1];
    if (k == 0) {
      mu0 = D0;
      mu1 = D1;
      mu[0] = D0;
      mu[1] = D1;
    } else {
      mu[2 * k] = 2 * D0 - mu0;
      mu[2 * k + 1] = 2 * D1 - mu1;
    }
  }
}

}  // namespace

extern "C" leo2d_status leo2d_kpm_dos_noalloc(const int64_t* rowptr, const int32_t* col,
                                              const float* val, int64_t n, int32_t poly_order,
                                              int32_t num_vectors, uint64_t seed,
                                              uint64_t first_vector, double* mu_out, void* stream) {
  auto bad = [](leo2d_status s, const char*) { return s; };
  if (!rowptr || !col || !val || !mu_out) return bad(LEO2D_ERR_BAD_ARG, "null pointer argument");
  if (n <= 0 || n >= (1ll << 31) - 1) return bad(LEO2D_ERR_BAD_ARG, "n must be in 1..2^31-2");
  if (poly_order < 4 || poly_order % 4 != 0)
    return bad(LEO2D_ERR_BAD_ARG, "poly_order must be a positive multiple of 4");
  if (num_vectors < 1) return bad(LEO2D_ERR_BAD_ARG, "num_vectors must be >= 1");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return bad(LEO2D_ERR_CUDA, "no current CUDA device");
  void* base = nullptr;
  {
    // once per device, with that device current
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      cudaError_t e = cudaGetSymbolAddress(&g_noalloc_ptr[dev], g_noalloc_scratch);
      if (e != cudaSuccess || !g_noalloc_ptr[dev]) {
        g_noalloc_ptr[dev] = nullptr;
        return bad(LEO2D_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
      }
    }
    base = g_noalloc_ptr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return bad(LEO2D_ERR_CUDA, "cannot query the device");
  const int steps = poly_order / 2;
  // widest block (8, 16 or 32 columns) whose working set fits the scratch array
  int cols = 0;
  unsigned grid = 0;
  size_t off_x1 = 0, off_part = 0, off_dots = 0;
  for (int c = 32; c >= 8; c /= 2) {
    StepShape s;
    s.cols = c;
    s.rows_per_item = 4;
    const int occ = std::max(1, occupancy(c, false));
    const int64_t item_rows = (int64_t)s.rows_per_item * (32 / c);
    const int64_t need = ((n + item_rows - 1) / item_rows + kWarps - 1) / kWarps;
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * occ, need));
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t xb = up((size_t)n * c * sizeof(float));
    const size_t pb = up((size_t)2 * g * 2 * c * sizeof(double));
    const size_t db = up((size_t)steps * 2 * c * sizeof(double));
    if (2 * xb + pb + db <= kNoAllocScratchBytes) {
      cols = c;
      grid = g;
      off_x1 = xb;
      off_part = 2 * xb;
      off_dots = 2 * xb + pb;
      break;
    }
  }
  if (cols == 0)
    return bad(LEO2D_ERR_BAD_ARG,
               "problem too large for the 32 MiB scratch array: n * 64 bytes plus moments must fit");
  unsigned char* sc = static_cast<unsigned char*>(base);
  float* x0 = reinterpret_cast<float*>(sc);
  float* x1 = reinterpret_cast<float*>(sc + off_x1);
  double* partials = reinterpret_cast<double*>(sc + off_part);
  double* dots = reinterpret_cast<double*>(sc + off_dots);
  const int vec_per_block = cols / 2;
  for (int v0 = 0; v0 < num_vectors; v0 += vec_per_block) {
    const int nv = std::min(vec_per_block, num_vectors - v0);
    const int64_t total = n * cols;
    k_fill_phase<float><<<(unsigned)std::min<int64_t>((total + 255) / 256, (int64_t)sms * 32), 256, 0, st>>>(
        n, cols, x0, seed, first_vector + v0, nv, nullptr);
    for (int k = 0; k < steps; ++k) {
      StepArgs<float> a;
      a.n = n;
      a.rowptr = rowptr;
      a.col = col;
      a.val = val;
      a.tn = k % 2 == 0 ? x0 : x1;
      a.tp = k % 2 == 0 ? x1 : x0;
      a.first = k == 0;
      a.alpha = 0.0f;
      a.tprev = nullptr;
      a.rows_per_item = 4;
      a.partials = partials + (size_t)(k % 2) * grid * 2 * cols;
      a.prev_partials = k == 0 ? nullptr : partials + (size_t)((k + 1) % 2) * grid * 2 * cols;
      a.prev_dots = k == 0 ? nullptr : dots + (size_t)(k - 1) * 2 * cols;
      switch (cols) {
        case 8: k_cheb_step<float, 1, 8><<<grid, kThreads, 0, st>>>(a); break;
        case 16: k_cheb_step<float, 1, 16><<<grid, kThreads, 0, st>>>(a); break;
        default: k_cheb_step<float, 1, 32><<<grid, kThreads, 0, st>>>(a); break;
      }
    }
    const double* last = partials + (size_t)((steps - 1) % 2) * grid * 2 * cols;
    double* last_dots = dots + (size_t)(steps - 1) * 2 * cols;
    const unsigned rg = (unsigned)std::min(2 * cols, 1024);
    switch (cols) {
      case 8: k_reduce_partials<8><<<rg, kThreads, 0, st>>>(last, last_dots, (int)grid); break;
      case 16: k_reduce_partials<16><<<rg, kThreads, 0, st>>>(last, last_dots, (int)grid); break;
      default: k_reduce_partials<32><<<rg, kThreads, 0, st>>>(last, last_dots, (int)grid); break;
    }
    k_dots_to_moments<<<(nv + 63) / 64, 64, 0, st>>>(dots, cols, steps, nv, mu_out + (size_t)v0 * poly_order,
                                                     poly_order);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return LEO2D_ERR_CUDA;
  }
  return LEO2D_OK;
}
