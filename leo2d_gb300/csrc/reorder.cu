// reorder.cu - locality ordering of the Hamiltonian for the recursion.
//
// The reference numbers orbitals sheet by sheet in grid-row order
// (Sheet::setIndex, src/geom/sheet.cpp:217-285), so the interlayer neighbours
// of a run of consecutive rows lie in a long strip of the other sheet. The
// recursion streams a permuted copy instead: orbitals of both sheets are
// grouped by square real-space patches (row-major patch order), which makes the
// T_n rows gathered by a row tile compact and L1-resident. Within a patch the
// orbitals go by sheet and then either by the reference index or (the curve
// ordering) along a Hilbert curve over 32 x 32 cells of the patch, so that any
// run of consecutive rows of one sheet is a compact cluster: 8 such rows share
// most of their neighbours (the 8-row blocks of rt_spmm.cu hold about 16 slots
// per row on twisted bilayers, against 18 with the reference index). The
// permutation is a stable sort of 32-bit keys (device LSD radix sort, 8-bit
// digits). Traces are invariant under the
// permutation; start vectors are generated from the reference index of each
// row, so moments equal those of the unpermuted matrix up to summation order.
#include <algorithm>
#include <cmath>

#include "csr.cuh"

using namespace leo2d;

namespace {

constexpr int kRsThreads = 256;
constexpr int kRsRounds = 16;
constexpr int kRsTile = kRsThreads * kRsRounds;
constexpr int kRsBins = 256;

__global__ void k_patch_keys(const double* __restrict__ pos, int64_t n, double x0, double y0,
                             double inv_s, int nx, uint32_t* __restrict__ keys,
                             int32_t* __restrict__ vals) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int px = (int)floor((pos[3 * k] - x0) * inv_s);
    const int py = (int)floor((pos[3 * k + 1] - y0) * inv_s);
    keys[k] = (uint32_t)(max(py, 0) * nx + max(px, 0));
    vals[k] = (int32_t)k;
  }
}

// Index of cell (x, y), 0 <= x, y < 32, along a Hilbert curve of the 32 x 32 cells.
__device__ __forceinline__ uint32_t hilbert32(uint32_t x, uint32_t y) {
  uint32_t d = 0;
  for (uint32_t s = 16; s > 0; s >>= 1) {
    const uint32_t rx = (x & s) ? 1u : 0u, ry = (y & s) ? 1u : 0u;
    d += s * s * ((3u * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = 31u - x;
        y = 31u - y;
      }
      const uint32_t tt = x;
      x = y;
      y = tt;
    }
  }
  return d;
}

// Curve keys: patch id (row-major) << 12 | sheet (2 bits) << 10 | Hilbert index of
// the orbital's 1/32-patch cell.
__global__ void k_curve_keys(const double* __restrict__ pos, const int32_t* __restrict__ grid4, int64_t n, double x0,
                             double y0, double patch, int nx, uint32_t* __restrict__ keys,
                             int32_t* __restrict__ vals) {
  const double inv_s = 1.0 / patch, inv_c = 32.0 / patch;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double dx = pos[3 * k] - x0, dy = pos[3 * k + 1] - y0;
    const int px = max((int)floor(dx * inv_s), 0), py = max((int)floor(dy * inv_s), 0);
    const int cx = min(max((int)floor(dx * inv_c) - 32 * px, 0), 31);
    const int cy = min(max((int)floor(dy * inv_c) - 32 * py, 0), 31);
    const uint32_t sheet = grid4 ? (uint32_t)min(max(grid4[4 * k + 3], 0), 3) : 0u;
    keys[k] = ((uint32_t)(py * nx + px) << 12) | (sheet << 10) | hilbert32((uint32_t)cx, (uint32_t)cy);
    vals[k] = (int32_t)k;
  }
}

__global__ void k_minmax_xy(const double* __restrict__ pos, int64_t n, double* __restrict__ out) {
  double xl = INFINITY, xh = -INFINITY, yl = INFINITY, yh = -INFINITY;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    xl = fmin(xl, pos[3 * k]); xh = fmax(xh, pos[3 * k]);
    yl = fmin(yl, pos[3 * k + 1]); yh = fmax(yh, pos[3 * k + 1]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    xl = fmin(xl, __shfl_down_sync(0xffffffffu, xl, o));
    xh = fmax(xh, __shfl_down_sync(0xffffffffu, xh, o));
    yl = fmin(yl, __shfl_down_sync(0xffffffffu, yl, o));
    yh = fmax(yh, __shfl_down_sync(0xffffffffu, yh, o));
  }
  if ((threadIdx.x & 31) == 0) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    out[4 * w] = xl; out[4 * w + 1] = xh; out[4 * w + 2] = yl; out[4 * w + 3] = yh;
  }
}

__global__ void k_rs_hist(const uint32_t* __restrict__ keys, int64_t n, int shift,
                          int64_t* __restrict__ hist, int nb) {
  __shared__ int cnt[kRsBins];
  for (int i = threadIdx.x; i < kRsBins; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t idx = base + r * kRsThreads + threadIdx.x;
    if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 255u], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRsBins; d += blockDim.x) hist[(int64_t)d * nb + blockIdx.x] = cnt[d];
}

// Stable scatter: keys of a tile keep their order within each digit.
__global__ void k_rs_scatter(const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin,
                             uint32_t* __restrict__ kout, int32_t* __restrict__ vout, int64_t n,
                             int shift, const int64_t* __restrict__ offs, int nb) {
  __shared__ int64_t base[kRsBins];
  __shared__ int running[kRsBins];
  __shared__ int wcnt[kRsThreads / 32][kRsBins];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < kRsBins; d += blockDim.x) {
    base[d] = offs[(int64_t)d * nb + blockIdx.x];
    running[d] = 0;
  }
  const int64_t tile0 = (int64_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsRounds; ++r) {
    for (int i = threadIdx.x; i < (kRsThreads / 32) * kRsBins; i += blockDim.x) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    const int64_t idx = tile0 + r * kRsThreads + threadIdx.x;
    const bool valid = idx < n;
    uint32_t key = 0;
    int32_t val = 0;
    int d = kRsBins;  // sentinel for lanes past the end
    if (valid) {
      key = kin[idx];
      val = vin[idx];
      d = (key >> shift) & 255u;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int wrank = __popc(peers & ((1u << lane) - 1u));
    if (valid && wrank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pre = 0;
      for (int w = 0; w < warp; ++w) pre += wcnt[w][d];
      const int64_t dst = base[d] + running[d] + pre + wrank;
      kout[dst] = key;
      vout[dst] = val;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kRsBins; t += blockDim.x) {
      int s = 0;
      for (int w = 0; w < kRsThreads / 32; ++w) s += wcnt[w][t];
      running[t] += s;
    }
    __syncthreads();
  }
}

__global__ void k_inverse_perm(const int32_t* __restrict__ new2old, int64_t n, int32_t* __restrict__ old2new) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x)
    old2new[new2old[r]] = (int32_t)r;
}

__global__ void k_perm_lengths(const int64_t* __restrict__ rp, const int32_t* __restrict__ new2old,
                               int64_t n, int64_t* __restrict__ len) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = new2old[r];
    len[r] = rp[k + 1] - rp[k];
  }
}

// One warp per permuted row: copy entries in their original order, columns renumbered.
__global__ void k_perm_fill(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                            const float* __restrict__ v32, const double* __restrict__ v64,
                            const float* __restrict__ im32, const int32_t* __restrict__ new2old,
                            const int32_t* __restrict__ old2new, const int64_t* __restrict__ prp, int64_t n,
                            int32_t* __restrict__ pcol, float* __restrict__ pv32, double* __restrict__ pv64,
                            float* __restrict__ pim32, uint2* __restrict__ pent) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
    const int64_t k = new2old[r];
    const int64_t b = rp[k], e = rp[k + 1], o = prp[r];
    for (int64_t i = b + lane; i < e; i += 32) {
      const int32_t c = old2new[col[i]];
      pcol[o + (i - b)] = c;
      pv32[o + (i - b)] = v32[i];
      pent[o + (i - b)] = make_uint2((unsigned)c, __float_as_uint(v32[i]));
      if (pv64) pv64[o + (i - b)] = v64[i];
      if (pim32) pim32[o + (i - b)] = im32[i];
    }
  }
}

}  // namespace

namespace leo2d {

void csr_build_reordered(leo2d_ctx* ctx, leo2d_csr* csr, double patch, bool with_fp64, bool curve) {
  const int curve_req = curve ? 1 : 0;
  csr_drop_tc(csr);
  csr_drop_rb(csr);
  csr_drop_rt(csr);
  const int64_t n = csr->n;
  LEO_REQUIRE(csr->pos.p, "locality ordering needs orbital positions");
  LEO_REQUIRE(patch > 0.5, "patch size must exceed 0.5 A");
  // bounding box
  const unsigned g = grid_for(n, 256, (int64_t)ctx->sm_count * 8);
  const int64_t nw = (int64_t)g * 8;
  DevBuf<double> mm(4 * nw);
  launch(ctx, "minmax_xy", [&] { k_minmax_xy<<<g, 256, 0, ctx->stream>>>(csr->pos.p, n, mm.p); });
  std::vector<double> h(4 * nw);
  d2h(ctx, h.data(), mm.p, h.size());
  ctx_sync(ctx);
  double xl = INFINITY, xh = -INFINITY, yl = INFINITY, yh = -INFINITY;
  for (int64_t w = 0; w < nw; ++w) {
    xl = std::fmin(xl, h[4 * w]); xh = std::fmax(xh, h[4 * w + 1]);
    yl = std::fmin(yl, h[4 * w + 2]); yh = std::fmax(yh, h[4 * w + 3]);
  }
  const int nx = (int)std::floor((xh - xl) / patch) + 1;
  const int ny = (int)std::floor((yh - yl) / patch) + 1;
  LEO_REQUIRE((int64_t)nx * ny < (1ll << 24), "too many patches");
  // the curve keys hold 20 bits of patch id
  if ((int64_t)nx * ny >= (1ll << 20)) curve = false;
  // keys and stable sort
  DevBuf<uint32_t> ka(n), kb(n);
  DevBuf<int32_t> va(n), vb(n);
  if (curve)
    launch(ctx, "patch_keys", [&] {
      k_curve_keys<<<grid_for(n, 256, (int64_t)ctx->sm_count * 32), 256, 0, ctx->stream>>>(
          csr->pos.p, csr->grid4.p, n, xl, yl, patch, nx, ka.p, va.p);
    });
  else
    launch(ctx, "patch_keys", [&] {
      k_patch_keys<<<grid_for(n, 256, (int64_t)ctx->sm_count * 32), 256, 0, ctx->stream>>>(
          csr->pos.p, n, xl, yl, 1.0 / patch, nx, ka.p, va.p);
    });
  const int nb = (int)((n + kRsTile - 1) / kRsTile);
  DevBuf<int64_t> hist((size_t)kRsBins * nb), offs((size_t)kRsBins * nb + 1);
  uint32_t *kin = ka.p, *kout = kb.p;
  int32_t *vin = va.p, *vout = vb.p;
  for (int shift = 0; shift < (curve ? 32 : 24); shift += 8) {
    launch(ctx, "rs_hist", [&] { k_rs_hist<<<nb, kRsThreads, 0, ctx->stream>>>(kin, n, shift, hist.p, nb); });
    exclusive_scan_i64(ctx, hist.p, offs.p, (int64_t)kRsBins * nb);
    launch(ctx, "rs_scatter", [&] {
      k_rs_scatter<<<nb, kRsThreads, 0, ctx->stream>>>(kin, vin, kout, vout, n, shift, offs.p, nb);
    });
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  // after the passes the sorted order is in (kin, vin)
  csr->new2old.alloc(n);
  csr->old2new.alloc(n);
  LEO_CUDA(cudaMemcpyAsync(csr->new2old.p, vin, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, ctx->stream));
  const unsigned gg = grid_for(n, 256, (int64_t)ctx->sm_count * 32);
  launch(ctx, "inverse_perm", [&] {
    k_inverse_perm<<<gg, 256, 0, ctx->stream>>>(csr->new2old.p, n, csr->old2new.p);
  });
  DevBuf<int64_t> len(n);
  launch(ctx, "perm_lengths", [&] {
    k_perm_lengths<<<gg, 256, 0, ctx->stream>>>(csr->rowptr.p, csr->new2old.p, n, len.p);
  });
  csr->prow.alloc(n + 1 + kCsrPad);
  LEO_CUDA(cudaMemsetAsync(csr->prow.p + n + 1, 0, kCsrPad * sizeof(int64_t), ctx->stream));
  exclusive_scan_i64(ctx, len.p, csr->prow.p, n);
  const int64_t nnz = csr->nnz;
  csr->pcol.alloc(nnz + kCsrPad);
  csr->pval32.alloc(nnz + kCsrPad);
  LEO_CUDA(cudaMemsetAsync(csr->pcol.p + nnz, 0, kCsrPad * sizeof(int32_t), ctx->stream));
  LEO_CUDA(cudaMemsetAsync(csr->pval32.p + nnz, 0, kCsrPad * sizeof(float), ctx->stream));
  csr->pent.alloc(nnz + kCsrPad);
  LEO_CUDA(cudaMemsetAsync(csr->pent.p + nnz, 0, kCsrPad * sizeof(uint2), ctx->stream));
  if (with_fp64) {
    csr->pval64.alloc(nnz + kCsrPad);
    LEO_CUDA(cudaMemsetAsync(csr->pval64.p + nnz, 0, kCsrPad * sizeof(double), ctx->stream));
  } else {
    csr->pval64.release();
  }
  if (csr->complex_h) {
    csr->pval_im32.alloc(nnz + kCsrPad);
    LEO_CUDA(cudaMemsetAsync(csr->pval_im32.p + nnz, 0, kCsrPad * sizeof(float), ctx->stream));
  }
  launch(ctx, "perm_fill", [&] {
    k_perm_fill<<<grid_for(n, 8, (int64_t)ctx->sm_count * 32), 256, 0, ctx->stream>>>(
        csr->rowptr.p, csr->col.p, csr->val32.p, csr->val64.p, csr->val_im32.p, csr->new2old.p, csr->old2new.p,
        csr->prow.p, n, csr->pcol.p, csr->pval32.p, with_fp64 ? csr->pval64.p : nullptr,
        csr->complex_h ? csr->pval_im32.p : nullptr, csr->pent.p);
  });
  ctx_sync(ctx);
  csr->reordered = true;
  csr->reorder_fp64 = with_fp64;
  csr->reorder_patch = patch;
  csr->reorder_curve = curve ? 1 : 0;
  csr->reorder_curve_req = curve_req;
  csr->perm_tile_rows = 0;
}

void csr_drop_reordered(leo2d_csr* csr) {
  csr_drop_tc(csr);
  csr_drop_rb(csr);
  csr_drop_rt(csr);
  csr->reordered = false;
  csr->reorder_fp64 = false;
  csr->new2old.release();
  csr->old2new.release();
  csr->prow.release();
  csr->pcol.release();
  csr->pval32.release();
  csr->pval64.release();
  csr->pent.release();
  csr->pval_im32.release();
}

}  // namespace leo2d
