// vacancy.cu - the matrix of a job with vacancies (removed orbitals).
//
// Replaces the vacancy path of Locality::generateRealH / generateCpxH
// (src/locality.cpp:2989-3016 relabelling, 3970-4010 and 4215-4220 skips,
// 4188 and 4305 renumbering): the reduced matrix is the full one without the
// rows of removed orbitals and without the entries in their columns, the kept
// orbitals renumbered in order (orbital i becomes i - removed orbitals below i).
// The full matrix is assembled once on the device; each vacancy job is then a
// compaction of it:
//   a keep flag per orbital, its exclusive scan (the new index of each kept
//   orbital and the kept count), the kept-entry count of each kept row, its
//   scan (the new row pointers), and one pass that copies each kept row's kept
//   entries in order (a warp per row, ballot compaction) with every value array
//   and the kept orbitals' positions and grid indices.
#include "csr.cuh"

using namespace leo2d;

namespace {

// keep[i] = 1 for every orbital, then 0 at each listed one (duplicates and
// indices outside [0, n) change nothing, as the reference's comparison loop)
__global__ void k_vac_keep(int64_t n, int64_t* __restrict__ keep) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    keep[i] = 1;
}
__global__ void k_vac_mark(int64_t n, const int64_t* __restrict__ orbitals, int64_t count,
                           int64_t* __restrict__ keep) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = orbitals[j];
    if (o >= 0 && o < n) keep[o] = 0;
  }
}

// newidx = exclusive scan of keep: orbital i is kept iff newidx[i + 1] > newidx[i]
__device__ __forceinline__ bool kept(const int64_t* newidx, int64_t i) { return newidx[i + 1] > newidx[i]; }

// cnt[newidx[r]] = kept entries of kept row r (a warp per row)
__global__ void k_vac_count(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                            const int64_t* __restrict__ newidx, int64_t* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
    if (!kept(newidx, r)) continue;
    int64_t c = 0;
    for (int64_t e = rowptr[r] + lane; e < rowptr[r + 1]; e += 32) c += kept(newidx, col[e]) ? 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[newidx[r]] = c;
  }
}

struct VacVals {
  const double* in[4];  // values, imaginary parts, dxH, dyH (null: absent)
  double* out[4];
};

// the kept entries of each kept row, in order, renumbered (a warp per row)
__global__ void k_vac_fill(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const int64_t* __restrict__ newidx, const int64_t* __restrict__ rp_out,
                           int32_t* __restrict__ col_out, const VacVals v) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
    if (!kept(newidx, r)) continue;
    int64_t o = rp_out[newidx[r]];
    const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
    for (int64_t b = e0; b < e1; b += 32) {  // warp-uniform bounds
      const int64_t e = b + lane;
      const int32_t c = e < e1 ? col[e] : 0;
      const bool k = e < e1 && kept(newidx, c);
      const unsigned m = __ballot_sync(0xffffffffu, k);
      if (k) {
        const int64_t d = o + __popc(m & lt);
        col_out[d] = (int32_t)newidx[c];
#pragma unroll
        for (int a = 0; a < 4; ++a)
          if (v.in[a]) v.out[a][d] = v.in[a][e];
      }
      o += __popc(m);
    }
  }
}

// positions and grid indices of the kept orbitals
__global__ void k_vac_rows(int64_t n, const int64_t* __restrict__ newidx, const double* __restrict__ pos,
                           const int32_t* __restrict__ grid4, double* __restrict__ pos_out,
                           int32_t* __restrict__ grid4_out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (!kept(newidx, i)) continue;
    const int64_t k = newidx[i];
    if (pos_out)
      for (int d = 0; d < 3; ++d) pos_out[3 * k + d] = pos[3 * i + d];
    if (grid4_out)
      for (int d = 0; d < 4; ++d) grid4_out[4 * k + d] = grid4[4 * i + d];
  }
}

}  // namespace

extern "C" leo2d_status leo2d_csr_remove_orbitals(leo2d_ctx* ctx, const leo2d_csr* src, const int64_t* orbitals,
                                                  int64_t count, leo2d_csr** out) {
  if (!ctx || !src || !out) return LEO2D_ERR_BAD_ARG;
  *out = nullptr;
  leo2d_csr* csr = nullptr;
  leo2d_status st = guard(ctx, [&] {
    LEO_REQUIRE(count >= 0 && (count == 0 || orbitals), "orbitals required when count > 0");
    LEO_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = src->n;
    DevBuf<int64_t> keep((size_t)n), newidx((size_t)n + 1);
    launch(ctx, "vac_keep", [&] {
      k_vac_keep<<<grid_for(n, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(n, keep.p);
    });
    if (count > 0) {
      DevBuf<int64_t> orb((size_t)count);
      h2d(ctx, orb.p, orbitals, count);
      launch(ctx, "vac_mark", [&] {
        k_vac_mark<<<grid_for(count, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(n, orb.p, count,
                                                                                                keep.p);
      });
      ctx_sync(ctx);  // orb is freed at the end of this scope
    }
    exclusive_scan_i64(ctx, keep.p, newidx.p, n);
    int64_t kept_n = 0;
    d2h(ctx, &kept_n, newidx.p + n, 1);
    ctx_sync(ctx);
    LEO_REQUIRE(kept_n >= 1, "every orbital is removed");

    csr = new leo2d_csr();
    csr->device = ctx->device;
    csr->n = kept_n;
    csr->flags = src->flags;
    csr->n_intra = src->n_intra;
    csr->n_inter = src->n_inter;
    csr->complex_h = src->complex_h;
    csr->has_geom = src->has_geom;
    csr->geom = src->geom;
    DevBuf<int64_t> cnt((size_t)kept_n);
    const unsigned rgrid = grid_for(n * 32, 256, (int64_t)ctx->sm_count * 16);
    launch(ctx, "vac_count", [&] {
      k_vac_count<<<rgrid, 256, 0, ctx->stream>>>(n, src->rowptr.p, src->col.p, newidx.p, cnt.p);
    });
    csr_alloc_rowptr(ctx, csr, kept_n);
    exclusive_scan_i64(ctx, cnt.p, csr->rowptr.p, kept_n);
    int64_t nnz = 0;
    d2h(ctx, &nnz, csr->rowptr.p + kept_n, 1);
    ctx_sync(ctx);
    csr->nnz = nnz;
    csr_alloc_entries(ctx, csr, nnz, src->dx64.p != nullptr);
    if (!src->dy64.p) csr->dy64.release();
    if (src->complex_h) {
      csr->val_im64.alloc(nnz + kCsrPad);
      LEO_CUDA(cudaMemsetAsync(csr->val_im64.p + nnz, 0, kCsrPad * sizeof(double), ctx->stream));
    }
    VacVals v{};
    v.in[0] = src->val64.p;
    v.out[0] = csr->val64.p;
    v.in[1] = src->complex_h ? src->val_im64.p : nullptr;
    v.out[1] = src->complex_h ? csr->val_im64.p : nullptr;
    v.in[2] = src->dx64.p;
    v.out[2] = src->dx64.p ? csr->dx64.p : nullptr;
    v.in[3] = src->dy64.p;
    v.out[3] = src->dy64.p ? csr->dy64.p : nullptr;
    launch(ctx, "vac_fill", [&] {
      k_vac_fill<<<rgrid, 256, 0, ctx->stream>>>(n, src->rowptr.p, src->col.p, newidx.p, csr->rowptr.p,
                                                 csr->col.p, v);
    });
    if (src->pos.p) csr->pos.alloc((size_t)3 * kept_n);
    if (src->grid4.p) csr->grid4.alloc((size_t)4 * kept_n);
    if (src->pos.p || src->grid4.p)
      launch(ctx, "vac_rows", [&] {
        k_vac_rows<<<grid_for(n, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
            n, newidx.p, src->pos.p, src->grid4.p, csr->pos.p, csr->grid4.p);
      });
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
