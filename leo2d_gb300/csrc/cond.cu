// cond.cu - Kubo conductivity moments and their transforms.
//
// Replaces Locality::computeCondKPM (src/locality.cpp:6348-6727) and
// Param_tools::conductivityTransform / matrixResponseTransform
// (src/params/param_tools.cpp:770-905).
//
// With D = dxH (D_ij = (x_i - x_j) H_ij, antisymmetric; J = iD up to sign) and a
// start vector r, the reference's moments are
//   C_nm = < D T_n(H~) a_0 , T_m(H~) r >,  a_0 = -D r,
// for r = e_t (locality.cpp:6471-6715), which equals <T_n D r | D T_m r> =
// <r| J T_n J T_m |r>; with random vectors r the same formula gives the trace
// mu_nm = Tr[J T_n J T_m] (stochastic estimate, new here).
// The reference recomputes D T_n a_0 for every m (O(P^2) SpMVs). Here each
// Chebyshev vector is built once:
//   B side: beta_m = T_m r          (one recursion, every vector kept)
//   A side: u_n    = D T_n a_0      (one recursion plus one D product per n)
// and C = U B^T is one GEMM over K = n_orbitals x columns, FP32 tiles with
// FP64 accumulation across K chunks. The reference never writes beta_{P-1}
// (its loop stops at P-2); in the per-target form that column is left 0.
//
// The trace form on a flake runs on the row-block step (32 columns per pass,
// locality-ordered rows) and stores no dxH: on a flake (dxH)_ij =
// (x_i - x_j) H~_ij exactly as assembled (geom.cu), so the A-side step forms
// D T_n from the gathers of the H~ T_n it computes anyway, with the rows' x
// positions as FP32 (hi, lo) pairs. U is held whole; B is built in chunks of
// moments, each chunk's product added into the columns of mu it covers.
#include <cmath>
#include <vector>

#include "kpm.cuh"
#include "tc_gemm.cuh"

using namespace leo2d;

namespace {

constexpr int kBM = 64, kBN = 64, kBK = 32;
constexpr int kGemmThreads = 256;
constexpr int kFlush = 16;  // BK steps between FP32 -> FP64 flushes (512 products)

// out[n][m] += sum_k A[n*lda + k*es] * B[m*ldb + k*es] over k in this block's chunk.
__global__ void __launch_bounds__(kGemmThreads) k_gemm_nt(const float* __restrict__ A,
                                                           const float* __restrict__ B, int M,
                                                           int64_t K, int64_t lda, int64_t ldb,
                                                           int64_t es, int64_t kchunk,
                                                           double* __restrict__ out) {
  __shared__ float As[kBK][kBM + 4];
  __shared__ float Bs[kBK][kBN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int n0 = blockIdx.y * kBM, m0 = blockIdx.x * kBN;
  const int64_t k_begin = (int64_t)blockIdx.z * kchunk;
  const int64_t k_end = min(K, k_begin + kchunk);
  float acc[4][4];
  double dacc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      acc[i][j] = 0.f;
      dacc[i][j] = 0.0;
    }
  int since = 0;
  for (int64_t k0 = k_begin; k0 < k_end; k0 += kBK) {
    // load: 64 rows x 32 k for A and B (8 elements per thread each)
    for (int e = threadIdx.x; e < kBM * kBK; e += kGemmThreads) {
      const int r = e / kBK, kk = e % kBK;
      const int64_t k = k0 + kk;
      const int na = n0 + r, mb = m0 + r;
      As[kk][r] = (na < M && k < k_end) ? A[(int64_t)na * lda + k * es] : 0.f;
      Bs[kk][r] = (mb < M && k < k_end) ? B[(int64_t)mb * ldb + k * es] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kBK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
    if (++since == kFlush) {
      since = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          dacc[i][j] += (double)acc[i][j];
          acc[i][j] = 0.f;
        }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + ty * 4 + i, m = m0 + tx * 4 + j;
      if (n < M && m < M) atomicAdd(&out[(int64_t)n * M + m], dacc[i][j] + (double)acc[i][j]);
    }
}

__global__ void k_scale(double* x, int64_t n, double s) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= s;
}

// 2-D DCT-III of 2 g_i g_j M_ij, g with the 1/sqrt(2) of matrixResponseTransform.
__global__ void k_cond_rows(const double* __restrict__ Min, int P, double* __restrict__ tmp) {
  const double pi = 3.141592653589793;
  const int64_t total = (int64_t)P * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / P), k = (int)(e % P);
    auto g = [&](int t) {
      return ((P - t) * cos((pi * t) / P) + sin((pi * t) / P) / tan(pi / P)) / (sqrt(2.0) * P);
    };
    const double gi = g(i);
    double acc = 0.0;
    const int64_t q = 2 * (int64_t)k + 1, den = 2 * (int64_t)P, period = 4 * (int64_t)P;
    for (int j = 0; j < P; ++j) {
      const double in = 2 * gi * g(j) * Min[(int64_t)i * P + j];
      const double c = j == 0 ? 1.0 : 2.0 * cospi((double)(((int64_t)j * q) % period) / (double)den);
      acc += in * c;
    }
    tmp[e] = acc;
  }
}

__global__ void k_cond_cols(const double* __restrict__ tmp, int P, double* __restrict__ out) {
  const int64_t total = (int64_t)P * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int k0 = (int)(e / P), k1 = (int)(e % P);
    double acc = 0.0;
    const int64_t q = 2 * (int64_t)k0 + 1, den = 2 * (int64_t)P, period = 4 * (int64_t)P;
    for (int i = 0; i < P; ++i) {
      const double c = i == 0 ? 1.0 : 2.0 * cospi((double)(((int64_t)i * q) % period) / (double)den);
      acc += tmp[(int64_t)i * P + k1] * c;
    }
    out[e] = acc;
  }
}

// sigma(E) = scale * sum_nm h_n h_m g_n g_m mu_nm T_n(x) T_m(x) / (pi^2 (1 - x^2)), h = 1, 2, 2, ...
__global__ void k_cond_sigma(const double* __restrict__ mu, int M, const double* __restrict__ E, int64_t nE,
                             double rescale, double center, double scale, double* __restrict__ out) {
  const double pi = 3.141592653589793;
  extern __shared__ double gsh[];
  for (int i = threadIdx.x; i < M; i += blockDim.x)
    gsh[i] = ((M - i) * cos((pi * i) / M) + sin((pi * i) / M) / tan(pi / M)) / M * (i == 0 ? 1.0 : 2.0);
  __syncthreads();
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nE; e += (int64_t)gridDim.x * blockDim.x) {
    const double x = (E[e] - center) / rescale;
    if (!(x > -1.0 && x < 1.0)) {
      out[e] = 0.0;
      continue;
    }
    double acc = 0.0, ta0 = 1.0, ta1 = x;
    for (int a = 0; a < M; ++a) {
      const double Ta = a == 0 ? 1.0 : (a == 1 ? x : 2.0 * x * ta1 - ta0);
      if (a >= 2) { ta0 = ta1; ta1 = Ta; }
      double row = 0.0, tb0 = 1.0, tb1 = x;
      for (int b = 0; b < M; ++b) {
        const double Tb = b == 0 ? 1.0 : (b == 1 ? x : 2.0 * x * tb1 - tb0);
        if (b >= 2) { tb0 = tb1; tb1 = Tb; }
        row += mu[(int64_t)a * M + b] * gsh[b] * Tb;
      }
      acc += row * gsh[a] * Ta;
    }
    out[e] = scale * acc / (pi * pi * (1.0 - x * x));
  }
}

// Whether the trace moments can take the row-block path: a flake assembled
// here (positions, no periodic images in dxH), the ordering allowed.
bool velocity_in_step(const leo2d_ctx* ctx, const leo2d_csr* csr) {
  return ctx->kubo_velocity != 0 && ctx->reorder != 0 && csr->has_geom && csr->geom.boundary_condition == 0 &&
         csr->pos.p != nullptr && csr->nnz > 0 && !csr->complex_h;
}

// acc[n][m] += sum over the vectors of <D T_n D r, T_m r> (note the sign: a_0
// = +D r here) on the row-block step; false when the row blocks do not fit
// (the stored-dxH path runs instead).
bool cond_trace_rows(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg, int P, double* acc) {
  leo2d_csr* m = const_cast<leo2d_csr*>(csr);
  StepShape s = choose_shape(ctx, csr, false, 32, 32, 0);
  s.rb = true;
  s.rt = false;  // the velocity step exists in the 4-row form only
  s.tc = false;
  s.rb_window = false;
  Recursion r;
  r.setup(ctx, csr, s, 1);
  // the velocity step's variant: the context's row-block settings where given,
  // else 16 warps, paired FMAs, 8 batches in flight
  StepShape sv = r.shape;
  sv.rb_warps = ctx->rb_warps > 0 ? ctx->rb_warps : 16;
  sv.rb_packed = ctx->rb_packed >= 0 ? ctx->rb_packed != 0 : true;
  sv.rb_unroll = ctx->rb_unroll > 0 ? ctx->rb_unroll : 8;
  if (sv.rb_warps != 16) {
    sv.rb_warps = 24;
    sv.rb_packed = false;
    sv.rb_unroll = 4;
  }
  if (!r.shape.rb || !r.use_perm || rb_stages(ctx, m, sv.rb_warps, true) < 2) return false;
  csr_build_rb_xs(ctx, m);
  // the B side's plain steps: the 8-row tensor-core step where it builds (the
  // 4-row step otherwise); its moment dots go to a scratch row nobody reads
  StepShape sb = choose_shape(ctx, csr, false, 32, 32, 0);
  sb.rb = false;
  sb.tc = false;
  sb.rt = ctx->kernel_variant == -1 || ctx->kernel_variant == 5;
  Recursion rt;
  if (sb.rt) rt.setup(ctx, csr, sb, 1);
  const bool b_rt = sb.rt && rt.shape.rt && rt.use_perm && m->rb_built;
  const size_t smem_v = rb_smem_bytes(ctx, m, sv.rb_warps, true);
  const unsigned grid_v = rb_grid(ctx, csr, sv.rb_warps);
  constexpr int C = 32;
  const int64_t n = csr->n;
  const size_t vec = (size_t)n * C;
  DevBuf<double> part((size_t)2 * std::max<unsigned>(ctx->sm_count, std::max(grid_v, r.grid)) * 2 * C);
  DevBuf<float> U((size_t)P * vec), ta(vec), tb(vec), junk(vec);
  // B-side moments held at once: the setting, else what fits next to U
  int64_t mc = P;
  if (ctx->kubo_chunk > 0) {
    mc = std::min<int64_t>(P, ctx->kubo_chunk);
  } else {
    size_t fr = 0, tot = 0;
    LEO_CUDA(cudaMemGetInfo(&fr, &tot));
    const size_t reserve = (size_t)3 << 30;  // GEMM partials, ordering and launch scratch
    const int64_t fit = fr > reserve ? (int64_t)((fr - reserve) / (vec * sizeof(float))) - 2 : 0;
    if (fit < P) mc = fit >= 256 ? fit / 256 * 256 : fit / 4 * 4;
    if (mc < 4) fail(LEO2D_ERR_OOM, "no room for the Kubo B-side vectors next to the A side");
  }
  DevBuf<float> Bc((size_t)(mc + 2) * vec);  // [carry T_{m0-2}, T_{m0-1}][T_{m0} ...]
  const int group = cfg->vector_kind == LEO2D_VEC_PHASE ? 2 : 1;
  const int per_block = C / group;
  for (int64_t v0 = 0; v0 < cfg->num_vectors; v0 += per_block) {
    const int nv = (int)std::min<int64_t>(per_block, cfg->num_vectors - v0);
    if (cfg->vector_kind == LEO2D_VEC_PHASE) fill_phase(ctx, r, cfg->seed, cfg->first_vector + v0, nv);
    else fill_gaussian(ctx, r, cfg->seed, cfg->first_vector + v0, nv);
    const float* X0 = reinterpret_cast<const float*>(r.x0.p);
    // a_0 = D r (its H~ r is not used)
    rb_launch_step(ctx, csr, sv, grid_v, smem_v, X0, junk.p, nullptr, 1, 1.f, part.p, nullptr, nullptr, ta.p);
    // A side: u_n = D T_n a_0 and T_{n+1} a_0 (over T_{n-1} a_0) from one launch
    float* cur = ta.p;
    float* nxt = tb.p;
    for (int k = 0; k < P; ++k) {
      rb_launch_step(ctx, csr, sv, grid_v, smem_v, cur, nxt, nullptr, k == 0 ? 1 : 0, k == 0 ? 1.f : 2.f, part.p,
                     nullptr, nullptr, U.p + (size_t)k * vec);
      std::swap(cur, nxt);
    }
    // B side in chunks: T_m in slot 2 + m - m0 (slots 0, 1: the previous chunk's last two)
    for (int64_t m0 = 0; m0 < P; m0 += mc) {
      const int64_t mn = std::min<int64_t>(mc, P - m0);
      auto slot = [&](int64_t mm) { return Bc.p + (size_t)(2 + mm - m0) * vec; };
      for (int64_t mm = m0; mm < m0 + mn; ++mm) {
        if (mm == 0)
          LEO_CUDA(cudaMemcpyAsync(slot(0), X0, vec * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
        else if (b_rt)
          rt_launch_step(ctx, csr, rt.shape, rt.grid, rt.dyn_smem, slot(mm - 1), slot(mm),
                         mm == 1 ? nullptr : slot(mm - 2), mm == 1 ? 1 : 0, mm == 1 ? 1.f : 2.f, part.p, nullptr,
                         nullptr);
        else if (mm == 1)
          rb_launch_step(ctx, csr, r.shape, r.grid, r.dyn_smem, slot(0), slot(1), nullptr, 1, 1.f, part.p,
                         nullptr, nullptr);
        else
          rb_launch_step(ctx, csr, r.shape, r.grid, r.dyn_smem, slot(mm - 1), slot(mm), slot(mm - 2), 0, 2.f,
                         part.p, nullptr, nullptr);
      }
      // mu[:, m0:m0+mn] += U B_chunk^T (three TF32 products, FP64 sums)
      tc_gemm_f32x3_acc(ctx, U.p, slot(m0), P, (int)mn, (int64_t)vec, acc + m0, P);
      if (m0 + mn < P) {
        LEO_CUDA(cudaMemcpyAsync(Bc.p, slot(m0 + mn - 2), vec * sizeof(float), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
        LEO_CUDA(cudaMemcpyAsync(Bc.p + vec, slot(m0 + mn - 1), vec * sizeof(float), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
      }
    }
  }
  return true;
}

void gemm(leo2d_ctx* ctx, const float* A, const float* Bm, int M, int64_t K, int64_t lda, int64_t ldb,
          int64_t es, double* out) {
  const int tiles = ((M + kBM - 1) / kBM) * ((M + kBN - 1) / kBN);
  int64_t splits = std::max<int64_t>(1, (int64_t)ctx->sm_count * 4 / std::max(tiles, 1));
  splits = std::min<int64_t>(splits, std::max<int64_t>(1, K / (kBK * kFlush)));
  int64_t kchunk = (K + splits - 1) / splits;
  kchunk = (kchunk + kBK - 1) / kBK * kBK;
  splits = (K + kchunk - 1) / kchunk;
  dim3 grid((M + kBN - 1) / kBN, (M + kBM - 1) / kBM, (unsigned)splits);
  launch(ctx, "cond_gemm", [&] {
    k_gemm_nt<<<grid, kGemmThreads, 0, ctx->stream>>>(A, Bm, M, K, lda, ldb, es, kchunk, out);
  });
}

}  // namespace

extern "C" {

leo2d_status leo2d_kpm_cond(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                            const int64_t* targets, int64_t num_targets, double* mu_out) {
  if (!ctx || !csr || !cfg || !mu_out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    const int P = cfg->poly_order;
    LEO_REQUIRE(P >= 4 && P % 4 == 0, "poly_order must be a positive multiple of 4");
    LEO_REQUIRE(cfg->precision == LEO2D_FP32 || cfg->precision == LEO2D_FP64, "unknown precision");
    LEO_REQUIRE(!csr->complex_h, "Kubo moments are built for a real Hamiltonian (no magnetic field)");
    const bool local = targets != nullptr;
    if (local) {
      LEO_REQUIRE(num_targets >= 1, "num_targets must be >= 1");
      for (int64_t t = 0; t < num_targets; ++t)
        LEO_REQUIRE(targets[t] >= 0 && targets[t] < csr->n, "target index out of range");
    } else {
      LEO_REQUIRE(cfg->num_vectors >= 1, "num_vectors must be >= 1");
      LEO_REQUIRE(cfg->vector_kind == LEO2D_VEC_PHASE || cfg->vector_kind == LEO2D_VEC_GAUSSIAN,
                  "trace conductivity takes random-phase or Gaussian vectors");
    }
    LEO_CUDA(cudaSetDevice(ctx->device));
    const bool fp64 = cfg->precision == LEO2D_FP64;
    LEO_REQUIRE(!fp64, "the Kubo recursion runs in FP32 (FP64 moments accumulate the GEMM)");
    if (!local && velocity_in_step(ctx, csr)) {
      DevBuf<double> acc((size_t)P * P);
      LEO_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(double) * P * P, ctx->stream));
      if (cond_trace_rows(ctx, csr, cfg, P, acc.p)) {
        ctx_check_status(ctx, "Kubo recursion");
        // a_0 = +D r above: the sign of -D r goes into the mean
        launch(ctx, "scale", [&] {
          k_scale<<<grid_for((int64_t)P * P, 256), 256, 0, ctx->stream>>>(acc.p, (int64_t)P * P,
                                                                          -1.0 / (double)cfg->num_vectors);
        });
        d2h(ctx, mu_out, acc.p, (size_t)P * P);
        ctx_sync(ctx);
        for (size_t i = 0; i < (size_t)P * P; ++i)
          if (!std::isfinite(mu_out[i])) fail(LEO2D_ERR_NONFINITE, "non-finite conductivity moment");
        return;
      }
    }
    LEO_REQUIRE(csr->dx64.p, "Kubo moments need dxH: build with LEO2D_CSR_WITH_DX");
    const int group = (!local && cfg->vector_kind == LEO2D_VEC_PHASE) ? 2 : 1;
    const int64_t total_cols = local ? num_targets : (int64_t)cfg->num_vectors * group;
    StepShape shape = choose_shape(ctx, csr, false, (int)std::min<int64_t>(total_cols, 8),
                                   cfg->block > 0 ? cfg->block : 8, cfg->rows_per_warp);
    Recursion r;
    r.allow_perm = false;
    r.setup(ctx, csr, shape, 1);
    const int C = shape.cols;
    const int64_t n = csr->n;
    const size_t vec = (size_t)n * C;
    DevBuf<float> U((size_t)P * vec), Bv((size_t)P * vec), a0(vec), t0(vec), t1(vec);
    DevBuf<double> acc((size_t)P * P);
    const int64_t out_sets = local ? num_targets : 1;
    std::vector<double> host((size_t)P * P);
    if (!local) LEO_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(double) * P * P, ctx->stream));
    const int per_block = local ? C : C / group;
    const int64_t items = local ? num_targets : cfg->num_vectors;
    for (int64_t v0 = 0; v0 < items; v0 += per_block) {
      const int nv = (int)std::min<int64_t>(per_block, items - v0);
      // start vectors r in x0
      if (local) fill_unit(ctx, r, targets + v0, nv);
      else if (cfg->vector_kind == LEO2D_VEC_PHASE) fill_phase(ctx, r, cfg->seed, cfg->first_vector + v0, nv);
      else fill_gaussian(ctx, r, cfg->seed, cfg->first_vector + v0, nv);
      const float* X0 = reinterpret_cast<const float*>(r.x0.p);
      // B side: beta_0 = r, beta_1 = H r, beta_{m+1} = 2 H beta_m - beta_{m-1}
      const int mb = local ? P - 1 : P;
      LEO_CUDA(cudaMemcpyAsync(Bv.p, X0, vec * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
      if (mb > 1) r.step(Bv.p, Bv.p + vec, nullptr, true, 1.0, 0);
      for (int m = 1; m + 1 < mb; ++m) r.step(Bv.p + m * vec, Bv.p + (m + 1) * vec, Bv.p + (m - 1) * vec, false, 2.0, 0);
      if (mb < P) LEO_CUDA(cudaMemsetAsync(Bv.p + (size_t)(P - 1) * vec, 0, vec * sizeof(float), ctx->stream));
      // A side: a_0 = -D r; u_n = D T_n a_0
      r.step(X0, a0.p, nullptr, true, -1.0, 1);
      float* tc = t0.p;  // T_n a_0
      float* tprev = t1.p;
      LEO_CUDA(cudaMemcpyAsync(tc, a0.p, vec * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
      for (int nidx = 0; nidx < P; ++nidx) {
        r.step(tc, U.p + (size_t)nidx * vec, nullptr, true, 1.0, 1);
        if (nidx + 1 < P) {
          // T_{n+1} a_0 written over T_{n-1} a_0
          r.step(tc, tprev, tprev, nidx == 0, nidx == 0 ? 1.0 : 2.0, 0);
          std::swap(tc, tprev);
        }
      }
      if (local) {
        for (int c = 0; c < nv; ++c) {
          LEO_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(double) * P * P, ctx->stream));
          gemm(ctx, U.p + c, Bv.p + c, P, n, (int64_t)vec, (int64_t)vec, C, acc.p);
          d2h(ctx, mu_out + (size_t)(v0 + c) * P * P, acc.p, (size_t)P * P);
          ctx_sync(ctx);
        }
      } else {
        // every column of the block: K = n x C; complex vectors add their two parts.
        // mu += U Bv^T on the tensor cores (three TF32 products, FP64 sum of ranges)
        tc_gemm_f32x3_acc(ctx, U.p, Bv.p, P, P, (int64_t)vec, acc.p);
      }
    }
    ctx_check_status(ctx, "Kubo recursion");
    if (!local) {
      launch(ctx, "scale", [&] {
        k_scale<<<grid_for((int64_t)P * P, 256), 256, 0, ctx->stream>>>(acc.p, (int64_t)P * P,
                                                                        1.0 / (double)cfg->num_vectors);
      });
      d2h(ctx, mu_out, acc.p, (size_t)P * P);
      ctx_sync(ctx);
    }
    (void)out_sets;
    for (size_t i = 0; i < (size_t)out_sets * P * P; ++i)
      if (!std::isfinite(mu_out[i])) fail(LEO2D_ERR_NONFINITE, "non-finite conductivity moment");
  });
}

leo2d_status leo2d_cond_transform(leo2d_ctx* ctx, const double* M, int32_t P, double* out) {
  if (!ctx || !M || !out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_REQUIRE(P >= 2, "poly_order >= 2 required");
    LEO_CUDA(cudaSetDevice(ctx->device));
    const int64_t pp = (int64_t)P * P;
    DevBuf<double> dm(pp), dt(pp), dout(pp);
    h2d(ctx, dm.p, M, pp);
    launch(ctx, "cond_rows", [&] { k_cond_rows<<<grid_for(pp, 128), 128, 0, ctx->stream>>>(dm.p, P, dt.p); });
    launch(ctx, "cond_cols", [&] { k_cond_cols<<<grid_for(pp, 128), 128, 0, ctx->stream>>>(dt.p, P, dout.p); });
    d2h(ctx, out, dout.p, pp);
    ctx_sync(ctx);
  });
}

leo2d_status leo2d_cond_sigma(leo2d_ctx* ctx, const double* mu, int32_t M, const double* energies,
                              int64_t num_energies, double rescale, double center, double scale,
                              double* sigma_out) {
  if (!ctx || !mu || !energies || !sigma_out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_REQUIRE(M >= 2 && num_energies >= 0, "bad sizes");
    LEO_REQUIRE(rescale > 0 && std::isfinite(rescale) && std::isfinite(center), "bad rescale/center");
    LEO_CUDA(cudaSetDevice(ctx->device));
    DevBuf<double> dmu((size_t)M * M), dE(std::max<int64_t>(num_energies, 1)),
        dout(std::max<int64_t>(num_energies, 1));
    h2d(ctx, dmu.p, mu, (size_t)M * M);
    h2d(ctx, dE.p, energies, num_energies);
    if (num_energies > 0)
      launch(ctx, "cond_sigma", [&] {
        k_cond_sigma<<<grid_for(num_energies, 128), 128, M * sizeof(double), ctx->stream>>>(
            dmu.p, M, dE.p, num_energies, rescale, center, scale, dout.p);
      });
    d2h(ctx, sigma_out, dout.p, num_energies);
    ctx_sync(ctx);
  });
}

}  // extern "C"
