// csr_api.cu - life cycle and host exchange of the device CSR, Gershgorin
// bounds and rescaling.
#include <cmath>
#include <cstring>

#include "csr.cuh"

using namespace leo2d;

namespace {

// Per-row Gershgorin interval of the stored matrix, reduced with min/max.
// A complex (Hermitian) matrix uses the moduli |H_ij| and the real diagonal.
__global__ void k_gershgorin(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                             const double* __restrict__ val, const double* __restrict__ im,
                             double* __restrict__ lo_out, double* __restrict__ hi_out) {
  double lo = INFINITY, hi = -INFINITY;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    double c = 0, rad = 0;
    for (int64_t i = rp[r]; i < rp[r + 1]; ++i) {
      if (col[i] == r) c += val[i];
      else rad += im ? hypot(val[i], im[i]) : fabs(val[i]);
    }
    lo = fmin(lo, c - rad);
    hi = fmax(hi, c + rad);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, o));
  }
  __shared__ double slo[32], shi[32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { slo[w] = lo; shi[w] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) { lo = fmin(lo, slo[i]); hi = fmax(hi, shi[i]); }
    lo_out[blockIdx.x] = lo;
    hi_out[blockIdx.x] = hi;
  }
}

// H <- (H + shift I) / rescale on the stored entries (diagonal gets the shift).
// (a complex matrix: the imaginary parts are divided, the shift is real)
// The division is a multiplication by the FP64 reciprocal (within an ulp of
// the quotient): FP64 division would bound the kernel on GB300's FP64 pipe.
__global__ void k_rescale(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                          double* __restrict__ val, double* __restrict__ im, double* __restrict__ dx,
                          double* __restrict__ dy, double inv, double shift) {
  // a warp per row, lanes over its entries (coalesced)
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
    for (int64_t i = rp[r] + lane; i < rp[r + 1]; i += 32) {
      val[i] = col[i] == r ? (val[i] + shift) * inv : val[i] * inv;
      if (im) im[i] = im[i] * inv;
      if (dx) dx[i] = dx[i] * inv;
      if (dy) dy[i] = dy[i] * inv;
    }
  }
}

}  // namespace

extern "C" {

leo2d_status leo2d_csr_destroy(leo2d_csr* csr) {
  if (!csr) return LEO2D_OK;
  cudaSetDevice(csr->device);
  delete csr;
  return LEO2D_OK;
}

leo2d_status leo2d_csr_info(const leo2d_csr* csr, int64_t* n, int64_t* nnz, int64_t* n_intra,
                            int64_t* n_inter) {
  if (!csr) return LEO2D_ERR_BAD_ARG;
  if (n) *n = csr->n;
  if (nnz) *nnz = csr->nnz;
  if (n_intra) *n_intra = csr->n_intra;
  if (n_inter) *n_inter = csr->n_inter;
  return LEO2D_OK;
}

leo2d_status leo2d_csr_download(leo2d_ctx* ctx, const leo2d_csr* csr, int64_t* rowptr, int32_t* col,
                                double* val, double* val_dx, double* val_dy) {
  if (!ctx || !csr) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_CUDA(cudaSetDevice(ctx->device));
    if (rowptr) d2h(ctx, rowptr, csr->rowptr.p, csr->n + 1);
    if (col) d2h(ctx, col, csr->col.p, csr->nnz);
    if (val) d2h(ctx, val, csr->val64.p, csr->nnz);
    if (val_dx) {
      LEO_REQUIRE(csr->dx64.p, "matrix was built without LEO2D_CSR_WITH_DX");
      d2h(ctx, val_dx, csr->dx64.p, csr->nnz);
    }
    if (val_dy) {
      LEO_REQUIRE(csr->dy64.p, "matrix was built without LEO2D_CSR_WITH_DX");
      d2h(ctx, val_dy, csr->dy64.p, csr->nnz);
    }
    ctx_sync(ctx);
  });
}

leo2d_status leo2d_csr_geometry(leo2d_ctx* ctx, const leo2d_csr* csr, int32_t* index_to_grid,
                                double* pos) {
  if (!ctx || !csr) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_CUDA(cudaSetDevice(ctx->device));
    if (index_to_grid) {
      LEO_REQUIRE(csr->grid4.p, "matrix has no geometry (uploaded without it)");
      d2h(ctx, index_to_grid, csr->grid4.p, 4 * csr->n);
    }
    if (pos) {
      LEO_REQUIRE(csr->pos.p, "matrix has no positions");
      d2h(ctx, pos, csr->pos.p, 3 * csr->n);
    }
    ctx_sync(ctx);
  });
}

leo2d_status leo2d_csr_upload(leo2d_ctx* ctx, int64_t n, int64_t nnz, const int64_t* rowptr,
                              const int32_t* col, const double* val, const double* val_dx,
                              const double* pos, leo2d_csr** out) {
  if (!ctx || !out) return LEO2D_ERR_BAD_ARG;
  *out = nullptr;
  leo2d_csr* csr = nullptr;
  leo2d_status st = guard(ctx, [&] {
    LEO_REQUIRE(n > 0 && n < (1ll << 31) - 1, "n must be in 1..2^31-2");
    LEO_REQUIRE(nnz >= 0, "nnz must be >= 0");
    LEO_REQUIRE(rowptr && (nnz == 0 || (col && val)), "rowptr/col/val required");
    LEO_REQUIRE(rowptr[0] == 0 && rowptr[n] == nnz, "rowptr must start at 0 and end at nnz");
    for (int64_t r = 0; r < n; ++r)
      LEO_REQUIRE(rowptr[r + 1] >= rowptr[r], "rowptr must be non-decreasing");
    for (int64_t i = 0; i < nnz; ++i) {
      LEO_REQUIRE(col[i] >= 0 && col[i] < n, "column index out of range");
      if (!std::isfinite(val[i])) fail(LEO2D_ERR_NONFINITE, "non-finite matrix value");
    }
    LEO_CUDA(cudaSetDevice(ctx->device));
    csr = new leo2d_csr();
    csr->device = ctx->device;
    csr->n = n;
    csr->nnz = nnz;
    csr_alloc_rowptr(ctx, csr, n);
    csr_alloc_entries(ctx, csr, nnz, false);
    h2d(ctx, csr->rowptr.p, rowptr, n + 1);
    h2d(ctx, csr->col.p, col, nnz);
    h2d(ctx, csr->val64.p, val, nnz);
    if (val_dx) {
      csr->dx64.alloc(nnz + kCsrPad);
      LEO_CUDA(cudaMemsetAsync(csr->dx64.p + nnz, 0, kCsrPad * sizeof(double), ctx->stream));
      h2d(ctx, csr->dx64.p, val_dx, nnz);
    }
    if (pos) {
      csr->pos.alloc(3 * n);
      h2d(ctx, csr->pos.p, pos, 3 * n);
    }
    csr_refresh_fp32(ctx, csr);
    ctx_sync(ctx);
  });
  if (st != LEO2D_OK) {
    delete csr;
    return st;
  }
  *out = csr;
  return LEO2D_OK;
}

leo2d_status leo2d_csr_download_imag(leo2d_ctx* ctx, const leo2d_csr* csr, double* val_im) {
  if (!ctx || !csr || !val_im) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_REQUIRE(csr->complex_h, "the matrix is real (built without a magnetic field)");
    LEO_CUDA(cudaSetDevice(ctx->device));
    d2h(ctx, val_im, csr->val_im64.p, (size_t)csr->nnz);
    ctx_sync(ctx);
  });
}

leo2d_status leo2d_csr_bounds(leo2d_ctx* ctx, const leo2d_csr* csr, double* emin, double* emax) {
  if (!ctx || !csr || !emin || !emax) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_CUDA(cudaSetDevice(ctx->device));
    const unsigned g = grid_for(csr->n, 256, (int64_t)ctx->sm_count * 4);
    DevBuf<double> lo(g), hi(g);
    launch(ctx, "gershgorin", [&] {
      k_gershgorin<<<g, 256, 0, ctx->stream>>>(csr->n, csr->rowptr.p, csr->col.p, csr->val64.p,
                                                csr->complex_h ? csr->val_im64.p : nullptr, lo.p, hi.p);
    });
    std::vector<double> hl(g), hh(g);
    d2h(ctx, hl.data(), lo.p, g);
    d2h(ctx, hh.data(), hi.p, g);
    ctx_sync(ctx);
    double a = INFINITY, b = -INFINITY;
    for (unsigned i = 0; i < g; ++i) {
      a = std::fmin(a, hl[i]);
      b = std::fmax(b, hh[i]);
    }
    *emin = a;
    *emax = b;
  });
}

leo2d_status leo2d_csr_rescale(leo2d_ctx* ctx, leo2d_csr* csr, double rescale, double shift) {
  if (!ctx || !csr) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_REQUIRE(rescale != 0.0 && std::isfinite(rescale) && std::isfinite(shift),
                "rescale must be finite and non-zero, shift finite");
    LEO_CUDA(cudaSetDevice(ctx->device));
    launch(ctx, "rescale", [&] {
      k_rescale<<<grid_for(csr->n * 32, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
          csr->n, csr->rowptr.p, csr->col.p, csr->val64.p, csr->complex_h ? csr->val_im64.p : nullptr,
          csr->dx64.p, csr->dy64.p, 1.0 / rescale, shift);
    });
    csr_refresh_fp32(ctx, csr);
    ctx_sync(ctx);
  });
}

}  // extern "C"
