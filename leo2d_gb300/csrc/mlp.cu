// mlp.cu - the learned control variate: a small MLP mapping a site's local
// stacking disregistry, twist, layer and sublattice to its first 256
// Chebyshev moments, trained and evaluated on the tensor cores.
//
// Network: 64 input features (16 used, zero padded) -> 256 -> 256 -> 256
// (GELU) -> 256 moments. BF16 weights and activations, FP32 accumulation
// (tc_gemm.cu), FP32 master weights, biases and Adam state.
//
// One training step (captured once into a CUDA graph, replayed per step):
//   gather a Philox-sampled minibatch X [B][64], T [B][256] (+ X^T)
//   forward: Z_l = A_l W_l^T + b_l  (A_0 = X, A_{l+1} = gelu(Z_l), Y = Z_3)
//   loss:    L = (1/B) sum_r sum_j w_j (Y - T)^2,  dZ_3 = (2/B) w (Y - T)
//   backward: dW_l = dZ_l^T A_l, db_l = colsum(dZ_l),
//             dZ_{l-1} = (dZ_l W_l) * gelu'(Z_{l-1})
//   Adam update of all parameters, refresh of the BF16 copies
//   (W_l [out][in] for the forward products, W_l^T [in][out] for dA).
// The reference has no learned component; the network only serves as a
// control variate for the stochastic trace (see the estimator in bench.py).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "csr.cuh"
#include "tc_gemm.cuh"

using namespace leo2d;

namespace {

constexpr int kIn = 64, kHid = 256, kOut = 256, kLayers = 4, kFeat = 16;
constexpr int kInDim[kLayers] = {kIn, kHid, kHid, kHid};
constexpr int64_t kChunk = 1 << 20;  // sites per inference pass
constexpr int kDwSplits = 32;        // K-range splits of the weight-gradient products

__device__ __forceinline__ uint32_t mix32(uint64_t a, uint64_t b) {
  // splitmix64 of (a, b): minibatch indices
  uint64_t z = a * 0x9E3779B97F4A7C15ull + b + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return (uint32_t)((z ^ (z >> 31)) >> 32);
}

// Site features from the disregistry (Hstruct::getShiftConfigs), twist,
// layer and sublattice; 16 used columns of 64.
__device__ __forceinline__ void site_features(double d0, double d1, float twist_deg, int layer, int sub,
                                              float* f) {
  const double tp = 6.283185307179586;
  f[0] = (float)cos(tp * d0);
  f[1] = (float)sin(tp * d0);
  f[2] = (float)cos(tp * d1);
  f[3] = (float)sin(tp * d1);
  f[4] = (float)cos(tp * (d0 + d1));
  f[5] = (float)sin(tp * (d0 + d1));
  f[6] = (float)cos(tp * (d0 - d1));
  f[7] = (float)sin(tp * (d0 - d1));
  f[8] = (float)cos(2 * tp * d0);
  f[9] = (float)sin(2 * tp * d0);
  f[10] = (float)cos(2 * tp * d1);
  f[11] = (float)sin(2 * tp * d1);
  f[12] = twist_deg / 3.0f;
  f[13] = (float)layer;
  f[14] = (float)sub;
  f[15] = 1.0f;
}

__global__ void k_features(int64_t n, int64_t first, const double* __restrict__ cfg,
                           const int32_t* __restrict__ grid4, float twist_deg, __nv_bfloat16* __restrict__ X,
                           float* __restrict__ Xf) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = first + r;
    float f[kFeat];
    site_features(cfg[2 * k], cfg[2 * k + 1], twist_deg, grid4[4 * k + 3], grid4[4 * k + 2], f);
    for (int c = 0; c < kIn; ++c) {
      const float v = c < kFeat ? f[c] : 0.0f;
      if (X) X[r * kIn + c] = __float2bfloat16_rn(v);
      if (Xf && c < kFeat) Xf[r * kFeat + c] = v;
    }
  }
}

// Features of selected orbitals rows[r] -> BF16 [n][64].
__global__ void k_features_at(int64_t n, const int64_t* __restrict__ rows, const double* __restrict__ cfg,
                              const int32_t* __restrict__ grid4, float twist_deg, __nv_bfloat16* __restrict__ X) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = rows[r];
    float f[kFeat];
    site_features(cfg[2 * k], cfg[2 * k + 1], twist_deg, grid4[4 * k + 3], grid4[4 * k + 2], f);
    for (int c = 0; c < kIn; ++c) X[r * kIn + c] = __float2bfloat16_rn(c < kFeat ? f[c] : 0.0f);
  }
}

// Host feature rows [n][F] (F <= 64, FP32) -> BF16 [n][64] and its transpose [64][ldt].
__global__ void k_pack_x(int64_t n, int F, const float* __restrict__ src, __nv_bfloat16* __restrict__ X,
                         __nv_bfloat16* __restrict__ Xt, int64_t ldt) {
  const int64_t total = n * kIn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / kIn;
    const int c = (int)(e % kIn);
    const __nv_bfloat16 v = __float2bfloat16_rn(c < F ? src[r * F + c] : 0.0f);
    X[e] = v;
    if (Xt) Xt[(int64_t)c * ldt + r] = v;
  }
}

// Minibatch: rows sampled (with replacement) by a hash of (seed, step, row).
__global__ void k_gather(int64_t n_train, int B, const __nv_bfloat16* __restrict__ Xall,
                         const float* __restrict__ Tall, const int64_t* __restrict__ step, uint64_t seed,
                         __nv_bfloat16* __restrict__ Xb, __nv_bfloat16* __restrict__ Xbt, float* __restrict__ Tb) {
  const uint64_t s = (uint64_t)*step;
  const int64_t total = (int64_t)B * (kIn + kOut);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / (kIn + kOut));
    const int c = (int)(e % (kIn + kOut));
    const int64_t src = (int64_t)(((uint64_t)mix32(seed ^ (s << 20), (uint64_t)r) * (uint64_t)n_train) >> 32);
    if (c < kIn) {
      const __nv_bfloat16 v = Xall[src * kIn + c];
      Xb[(int64_t)r * kIn + c] = v;
      Xbt[(int64_t)c * B + r] = v;
    } else {
      Tb[(int64_t)r * kOut + (c - kIn)] = Tall[src * kOut + (c - kIn)];
    }
  }
}

// dY = (2/n) w (Y - T) -> BF16 [n][256], its transpose, FP32; per-block loss sums.
__global__ void __launch_bounds__(256) k_loss(int n, const float* __restrict__ Y, const float* __restrict__ T,
                                              const float* __restrict__ w, __nv_bfloat16* __restrict__ dZ,
                                              __nv_bfloat16* __restrict__ dZt, int64_t ldt, float* __restrict__ dZ32,
                                              double* __restrict__ part) {
  __shared__ double red[256];
  double acc = 0.0;
  const int64_t total = (int64_t)n * kOut;
  const float scale = 2.0f / (float)n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / kOut), j = (int)(e % kOut);
    const float d = Y[e] - T[e];
    const float g = scale * w[j] * d;
    acc += (double)w[j] * (double)d * (double)d;
    dZ32[e] = g;
    const __nv_bfloat16 b = __float2bfloat16_rn(g);
    dZ[e] = b;
    dZt[(int64_t)j * ldt + r] = b;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_loss_final(const double* __restrict__ part, int nb, int n, const int64_t* __restrict__ step,
                             double* __restrict__ hist, int64_t hist_cap, double* __restrict__ last) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += part[b];
  s /= (double)n;
  *last = s;
  const int64_t t = step ? *step : 0;
  if (hist && t < hist_cap) hist[t] = s;
}

// Column sums of x [n][256] (FP32) in two fixed-order passes.
__global__ void __launch_bounds__(256) k_colsum_part(int n, int rows_per_block, const float* __restrict__ x,
                                                     float* __restrict__ part) {
  const int j = threadIdx.x;
  const int r0 = blockIdx.x * rows_per_block, r1 = min(n, r0 + rows_per_block);
  float s = 0.0f;
  for (int r = r0; r < r1; ++r) s += x[(int64_t)r * kOut + j];
  part[(int64_t)blockIdx.x * kOut + j] = s;
}
__global__ void __launch_bounds__(256) k_colsum_final(const float* __restrict__ part, int nb, float* __restrict__ out) {
  const int j = threadIdx.x;
  float s = 0.0f;
  for (int b = 0; b < nb; ++b) s += part[(int64_t)b * kOut + j];
  out[j] = s;
}

__global__ void k_adam(int64_t np, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, const int64_t* __restrict__ step, float lr, float b1, float b2,
                       float eps) {
  const double t = (double)(*step + 1);
  const float c1 = (float)(1.0 - pow((double)b1, t)), c2 = (float)(1.0 - pow((double)b2, t));
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_step_inc(int64_t* step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1;
}

// W [out][in] FP32 -> BF16 [out][in] and (optionally) BF16 [in][out].
__global__ void k_refresh(int out, int in, const float* __restrict__ W, __nv_bfloat16* __restrict__ wt,
                          __nv_bfloat16* __restrict__ wn) {
  const int64_t total = (int64_t)out * in;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int o = (int)(e / in), i = (int)(e % in);
    const __nv_bfloat16 b = __float2bfloat16_rn(W[e]);
    wt[e] = b;
    if (wn) wn[(int64_t)i * out + o] = b;
  }
}

__global__ void k_sum_partials(const double* __restrict__ part, int nb, double* __restrict__ out, int accumulate) {
  const int j = threadIdx.x;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += part[(int64_t)b * kOut + j];
  out[j] = accumulate ? out[j] + s : s;
}

uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

struct leo2d_mlp {
  leo2d_ctx* ctx = nullptr;
  int64_t np = 0;
  int64_t w_off[kLayers], b_off[kLayers];
  DevBuf<float> p, g, m, v, lw;
  DevBuf<__nv_bfloat16> wt[kLayers], wn[kLayers];
  DevBuf<int64_t> step;
  // training workspace (batch B)
  int B = 0;
  DevBuf<__nv_bfloat16> Xb, Xbt, A[kLayers], At[kLayers], dZ[2], dZt[2];
  DevBuf<float> Tb, Z[kLayers], Y, dZ32[2], cs_part, dw_split;
  DevBuf<double> loss_part, loss_last, loss_hist;
  int64_t hist_cap = 0;
  CUtensorMap tX, tA[kLayers], tWt[kLayers], tWn[kLayers], tXt, tAt[kLayers], tdZ[2], tdZt[2];
  // training set
  int64_t n_train = 0;
  DevBuf<__nv_bfloat16> Xall;
  DevBuf<float> Tall;
  cudaGraphExec_t graph = nullptr;
  uint64_t graph_seed = 0;
  float graph_lr = 0.f;
  ~leo2d_mlp() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

namespace {

void refresh_bf16(leo2d_mlp* M) {
  leo2d_ctx* ctx = M->ctx;
  for (int l = 0; l < kLayers; ++l) {
    const int in = kInDim[l];
    launch(ctx, "mlp_refresh", [&] {
      k_refresh<<<grid_for((int64_t)kHid * in, 256, ctx->sm_count * 8), 256, 0, ctx->stream>>>(
          kHid, in, M->p.p + M->w_off[l], M->wt[l].p, l > 0 ? M->wn[l].p : nullptr);
    });
  }
}

void ensure_batch(leo2d_mlp* M, int B) {
  if (M->B == B) return;
  LEO_REQUIRE(B >= 64 && B % 64 == 0 && B <= (1 << 20), "batch must be a multiple of 64 in [64, 2^20]");
  if (M->graph) {
    cudaGraphExecDestroy(M->graph);
    M->graph = nullptr;
  }
  M->B = B;
  M->Xb.alloc((size_t)B * kIn);
  M->Xbt.alloc((size_t)kIn * B);
  M->Tb.alloc((size_t)B * kOut);
  M->Y.alloc((size_t)B * kOut);
  for (int l = 0; l < kLayers; ++l) {
    if (l > 0) {
      M->A[l].alloc((size_t)B * kHid);
      M->At[l].alloc((size_t)kHid * B);
    }
    if (l < kLayers - 1) M->Z[l].alloc((size_t)B * kHid);
  }
  for (int i = 0; i < 2; ++i) {
    M->dZ[i].alloc((size_t)B * kHid);
    M->dZt[i].alloc((size_t)kHid * B);
    M->dZ32[i].alloc((size_t)B * kHid);
  }
  M->dw_split.alloc((size_t)kDwSplits * kHid * kHid);
  const int cs_blocks = (B + 63) / 64;
  M->cs_part.alloc((size_t)cs_blocks * kOut);
  M->loss_part.alloc(1024);
  M->loss_last.alloc(1);
  make_tmap_bf16(&M->tX, M->Xb.p, B, kIn, kGemmBM);
  make_tmap_bf16(&M->tXt, M->Xbt.p, kIn, B, 256);
  for (int l = 1; l < kLayers; ++l) {
    make_tmap_bf16(&M->tA[l], M->A[l].p, B, kHid, kGemmBM);
    make_tmap_bf16(&M->tAt[l], M->At[l].p, kHid, B, 256);
  }
  for (int i = 0; i < 2; ++i) {
    make_tmap_bf16(&M->tdZ[i], M->dZ[i].p, B, kHid, kGemmBM);
    make_tmap_bf16(&M->tdZt[i], M->dZt[i].p, kHid, B, kGemmBM);
  }
}

// Forward over the first n rows of Xb (n <= B); Y [n][256] FP32.
void forward_train(leo2d_mlp* M, int n) {
  leo2d_ctx* ctx = M->ctx;
  for (int l = 0; l < kLayers; ++l) {
    GemmArgs g{};
    g.M = n;
    g.N = kHid;
    g.K = kInDim[l];
    g.bias = M->p.p + M->b_off[l];
    g.status = ctx->status.p;
    const CUtensorMap& ta = l == 0 ? M->tX : M->tA[l];
    if (l < kLayers - 1) {
      g.zout = M->Z[l].p;
      g.out_bf16 = M->A[l + 1].p;
      g.out_bf16_t = M->At[l + 1].p;
      g.ld_t = M->B;
      tc_gemm(ctx, kEpiBiasGelu, ta, M->tWt[l], g);
    } else {
      g.out_f32 = M->Y.p;
      tc_gemm(ctx, kEpiBias, ta, M->tWt[l], g);
    }
  }
}

// Loss on rows [0, n) against Tb, then gradients of every parameter into g.
void backward_train(leo2d_mlp* M, int n) {
  leo2d_ctx* ctx = M->ctx;
  const int B = M->B;
  const int lb = (int)std::min<int64_t>(1024, grid_for((int64_t)n * kOut, 256));
  launch(ctx, "mlp_loss", [&] {
    k_loss<<<lb, 256, 0, ctx->stream>>>(n, M->Y.p, M->Tb.p, M->lw.p, M->dZ[1].p, M->dZt[1].p, B, M->dZ32[1].p,
                                        M->loss_part.p);
  });
  launch(ctx, "mlp_loss", [&] {
    k_loss_final<<<1, 32, 0, ctx->stream>>>(M->loss_part.p, lb, n, M->step.p, M->loss_hist.p, M->hist_cap,
                                            M->loss_last.p);
  });
  int cur = 1;  // dZ of layer l lives in buffer `cur`
  for (int l = kLayers - 1; l >= 0; --l) {
    // bias gradient
    const int rpb = 64, nb = (n + rpb - 1) / rpb;
    launch(ctx, "mlp_colsum", [&] {
      k_colsum_part<<<nb, 256, 0, ctx->stream>>>(n, rpb, M->dZ32[cur].p, M->cs_part.p);
    });
    launch(ctx, "mlp_colsum", [&] {
      k_colsum_final<<<1, 256, 0, ctx->stream>>>(M->cs_part.p, nb, M->g.p + M->b_off[l]);
    });
    // weight gradient dW_l [out][in] = dZ_l^T A_l
    {
      GemmArgs g{};
      g.M = kHid;
      g.N = kInDim[l];
      g.K = n;
      g.out_f32 = M->g.p + M->w_off[l];
      g.status = ctx->status.p;
      // K = n rows: split over up to 32 work items per output tile
      g.k_splits = std::max(1, std::min(kDwSplits, n / 256));
      g.split_buf = M->dw_split.p;
      tc_gemm(ctx, kEpiF32, M->tdZt[cur], l == 0 ? M->tXt : M->tAt[l], g);
    }
    if (l == 0) break;
    // dZ_{l-1} = (dZ_l W_l) * gelu'(Z_{l-1})
    {
      const int nxt = cur ^ 1;
      GemmArgs g{};
      g.M = n;
      g.N = kHid;
      g.K = kHid;
      g.zin = M->Z[l - 1].p;
      g.out_f32 = M->dZ32[nxt].p;
      g.out_bf16 = M->dZ[nxt].p;
      g.out_bf16_t = M->dZt[nxt].p;
      g.ld_t = B;
      g.status = ctx->status.p;
      tc_gemm(ctx, kEpiGeluBwd, M->tdZ[cur], M->tWn[l], g);
      cur = nxt;
    }
  }
}

void adam_update(leo2d_mlp* M, float lr) {
  leo2d_ctx* ctx = M->ctx;
  launch(ctx, "mlp_adam", [&] {
    k_adam<<<grid_for(M->np, 256, ctx->sm_count * 4), 256, 0, ctx->stream>>>(M->np, M->p.p, M->g.p, M->m.p, M->v.p,
                                                                             M->step.p, lr, 0.9f, 0.999f, 1e-8f);
  });
  refresh_bf16(M);
  launch(ctx, "mlp_step", [&] { k_step_inc<<<1, 32, 0, ctx->stream>>>(M->step.p); });
}

void train_step_enqueue(leo2d_mlp* M, uint64_t seed, float lr) {
  leo2d_ctx* ctx = M->ctx;
  const int B = M->B;
  launch(ctx, "mlp_gather", [&] {
    k_gather<<<grid_for((int64_t)B * (kIn + kOut), 256, ctx->sm_count * 8), 256, 0, ctx->stream>>>(
        M->n_train, B, M->Xall.p, M->Tall.p, M->step.p, seed, M->Xb.p, M->Xbt.p, M->Tb.p);
  });
  forward_train(M, B);
  backward_train(M, B);
  adam_update(M, lr);
}

void upload_x(leo2d_mlp* M, const float* x, int64_t n, int F) {
  leo2d_ctx* ctx = M->ctx;
  DevBuf<float> src((size_t)n * F);
  h2d(ctx, src.p, x, (size_t)n * F);
  launch(ctx, "mlp_pack", [&] {
    k_pack_x<<<grid_for(n * kIn, 256, ctx->sm_count * 8), 256, 0, ctx->stream>>>(n, F, src.p, M->Xb.p, M->Xbt.p,
                                                                                 M->B);
  });
  ctx_sync(ctx);
}

// Forward of `n` rows whose BF16 features sit in X (row-major [n][64]): either
// Y [n][256] FP32, or the column sums (FP64). By default one fused launch keeps
// every activation on chip (mlp_fused.cu); option mlp_fused = 0 runs one GEMM
// per layer over chunks of kChunk rows, with the activations in HBM.
void infer_rows(leo2d_mlp* M, const __nv_bfloat16* X, int64_t n, float* Y, double* sums_dev) {
  leo2d_ctx* ctx = M->ctx;
  if (ctx->mlp_fused) {
    CUtensorMap tx;
    make_tmap_bf16(&tx, X, n, kIn, kGemmBM);
    const float* bias[kLayers];
    for (int l = 0; l < kLayers; ++l) bias[l] = M->p.p + M->b_off[l];
    mlp_forward_fused(ctx, tx, M->tWt, bias, n, Y, sums_dev);
    return;
  }
  const int64_t chunk = std::min<int64_t>(kChunk, n);
  DevBuf<__nv_bfloat16> h0((size_t)chunk * kHid), h1((size_t)chunk * kHid);
  const int grid = tc_gemm_grid(ctx, (int)chunk, kOut);
  DevBuf<double> part((size_t)grid * kOut);
  bool first = true;
  for (int64_t r0 = 0; r0 < n; r0 += chunk) {
    const int rows = (int)std::min<int64_t>(chunk, n - r0);
    CUtensorMap tx, th0, th1;
    make_tmap_bf16(&tx, X + r0 * kIn, rows, kIn, kGemmBM);
    make_tmap_bf16(&th0, h0.p, rows, kHid, kGemmBM);
    make_tmap_bf16(&th1, h1.p, rows, kHid, kGemmBM);
    const CUtensorMap* in_map[kLayers] = {&tx, &th0, &th1, &th0};
    __nv_bfloat16* out_buf[kLayers - 1] = {h0.p, h1.p, h0.p};
    for (int l = 0; l < kLayers; ++l) {
      GemmArgs g{};
      g.M = rows;
      g.N = kHid;
      g.K = kInDim[l];
      g.bias = M->p.p + M->b_off[l];
      g.status = ctx->status.p;
      if (l < kLayers - 1) {
        g.out_bf16 = out_buf[l];
        tc_gemm(ctx, kEpiBiasGelu, *in_map[l], M->tWt[l], g);
      } else if (Y) {
        g.out_f32 = Y + r0 * kOut;
        tc_gemm(ctx, kEpiBias, *in_map[l], M->tWt[l], g);
      } else {
        g.colsum = part.p;
        const int gr = tc_gemm_grid(ctx, rows, kOut);
        tc_gemm(ctx, kEpiBias, *in_map[l], M->tWt[l], g);
        launch(ctx, "mlp_sum", [&] {
          k_sum_partials<<<1, kOut, 0, ctx->stream>>>(part.p, gr, sums_dev, first ? 0 : 1);
        });
      }
    }
    first = false;
    ctx_sync(ctx);  // the chunk's tensor maps and buffers are reused by the next chunk
  }
}

}  // namespace

// ---------------------------------------------------------------- C ABI

extern "C" {

int64_t leo2d_mlp_param_count(void) {
  return (int64_t)kHid * kIn + kHid + (int64_t)(kLayers - 1) * ((int64_t)kHid * kHid + kHid);
}

leo2d_status leo2d_mlp_create(leo2d_ctx* ctx, uint64_t seed, leo2d_mlp** out) {
  if (!ctx || !out) return LEO2D_ERR_BAD_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    LEO_CUDA(cudaSetDevice(ctx->device));
    auto M = std::make_unique<leo2d_mlp>();
    M->ctx = ctx;
    int64_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
      M->w_off[l] = off;
      off += (int64_t)kHid * kInDim[l];
      M->b_off[l] = off;
      off += kHid;
    }
    M->np = off;
    // He-uniform weights on the used inputs (layer 0: the 16 feature columns),
    // a narrower output layer, zero biases; splitmix64 stream from `seed`
    std::vector<float> h((size_t)off, 0.0f);
    uint64_t st = seed;
    for (int l = 0; l < kLayers; ++l) {
      const int in_used = l == 0 ? kFeat : kInDim[l];
      const double a = l == kLayers - 1 ? std::sqrt(1.0 / in_used) : std::sqrt(6.0 / in_used);
      for (int o = 0; o < kHid; ++o)
        for (int i = 0; i < kInDim[l]; ++i) {
          const double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
          h[M->w_off[l] + (size_t)o * kInDim[l] + i] = i < in_used ? (float)((2.0 * u - 1.0) * a) : 0.0f;
        }
    }
    M->p.alloc(off);
    M->g.alloc(off);
    M->m.alloc(off);
    M->v.alloc(off);
    h2d(ctx, M->p.p, h.data(), (size_t)off);
    LEO_CUDA(cudaMemsetAsync(M->m.p, 0, sizeof(float) * off, ctx->stream));
    LEO_CUDA(cudaMemsetAsync(M->v.p, 0, sizeof(float) * off, ctx->stream));
    LEO_CUDA(cudaMemsetAsync(M->g.p, 0, sizeof(float) * off, ctx->stream));
    std::vector<float> ones(kOut, 1.0f);
    M->lw.alloc(kOut);
    h2d(ctx, M->lw.p, ones.data(), kOut);
    M->step.alloc(1);
    LEO_CUDA(cudaMemsetAsync(M->step.p, 0, sizeof(int64_t), ctx->stream));
    for (int l = 0; l < kLayers; ++l) {
      M->wt[l].alloc((size_t)kHid * kInDim[l]);
      make_tmap_bf16(&M->tWt[l], M->wt[l].p, kHid, kInDim[l], 256);
      if (l > 0) {
        M->wn[l].alloc((size_t)kInDim[l] * kHid);
        make_tmap_bf16(&M->tWn[l], M->wn[l].p, kInDim[l], kHid, 256);
      }
    }
    refresh_bf16(M.get());
    tc_gemm_prepare(ctx);
    ctx_sync(ctx);
    *out = M.release();
  });
}

leo2d_status leo2d_mlp_destroy(leo2d_mlp* M) {
  if (!M) return LEO2D_OK;
  cudaSetDevice(M->ctx->device);
  delete M;
  return LEO2D_OK;
}

leo2d_status leo2d_mlp_get_params(leo2d_mlp* M, float* out) {
  if (!M || !out) return LEO2D_ERR_BAD_ARG;
  return guard(M->ctx, [&] {
    d2h(M->ctx, out, M->p.p, (size_t)M->np);
    ctx_sync(M->ctx);
  });
}

leo2d_status leo2d_mlp_set_params(leo2d_mlp* M, const float* in) {
  if (!M || !in) return LEO2D_ERR_BAD_ARG;
  return guard(M->ctx, [&] {
    for (int64_t i = 0; i < M->np; ++i) LEO_REQUIRE(std::isfinite(in[i]), "parameters must be finite");
    h2d(M->ctx, M->p.p, in, (size_t)M->np);
    refresh_bf16(M);
    ctx_sync(M->ctx);
  });
}

leo2d_status leo2d_mlp_set_loss_weights(leo2d_mlp* M, const float* w) {
  if (!M || !w) return LEO2D_ERR_BAD_ARG;
  return guard(M->ctx, [&] {
    h2d(M->ctx, M->lw.p, w, kOut);
    ctx_sync(M->ctx);
  });
}

leo2d_status leo2d_mlp_grad(leo2d_mlp* M, const float* x, int32_t F, const float* t, int64_t n, double* loss,
                            float* grad) {
  if (!M || !x || !t || !loss || !grad) return LEO2D_ERR_BAD_ARG;
  leo2d_ctx* ctx = M->ctx;
  return guard(ctx, [&] {
    LEO_REQUIRE(F >= 1 && F <= kIn, "feature count must be 1..64");
    LEO_REQUIRE(n >= 64 && n % 64 == 0 && n <= (1 << 16), "n must be a multiple of 64 in [64, 65536]");
    LEO_CUDA(cudaSetDevice(ctx->device));
    ensure_batch(M, (int)n);
    upload_x(M, x, n, F);
    h2d(ctx, M->Tb.p, t, (size_t)n * kOut);
    if (!M->loss_hist.p) M->loss_hist.alloc(1);
    forward_train(M, (int)n);
    backward_train(M, (int)n);
    d2h(ctx, loss, M->loss_last.p, 1);
    d2h(ctx, grad, M->g.p, (size_t)M->np);
    ctx_check_status(ctx, "MLP gradient");
  });
}

leo2d_status leo2d_mlp_train(leo2d_mlp* M, const float* x, int32_t F, const float* t, int64_t n, int32_t steps,
                             int32_t batch, float lr, uint64_t seed, double* loss_hist) {
  if (!M || !x || !t) return LEO2D_ERR_BAD_ARG;
  leo2d_ctx* ctx = M->ctx;
  return guard(ctx, [&] {
    LEO_REQUIRE(F >= 1 && F <= kIn, "feature count must be 1..64");
    LEO_REQUIRE(n >= 1, "empty training set");
    LEO_REQUIRE(steps >= 0, "steps must be >= 0");
    LEO_REQUIRE(lr > 0 && std::isfinite(lr), "learning rate must be positive");
    LEO_CUDA(cudaSetDevice(ctx->device));
    ensure_batch(M, batch);
    // training set: BF16 features [n][64], FP32 targets [n][256]
    {
      DevBuf<float> src((size_t)n * F);
      h2d(ctx, src.p, x, (size_t)n * F);
      M->Xall.alloc((size_t)n * kIn);
      launch(ctx, "mlp_pack", [&] {
        k_pack_x<<<grid_for(n * kIn, 256, ctx->sm_count * 8), 256, 0, ctx->stream>>>(n, F, src.p, M->Xall.p,
                                                                                     nullptr, 0);
      });
      M->Tall.alloc((size_t)n * kOut);
      h2d(ctx, M->Tall.p, t, (size_t)n * kOut);
      M->n_train = n;
      ctx_sync(ctx);
    }
    int64_t t0 = 0;
    d2h(ctx, &t0, M->step.p, 1);
    ctx_sync(ctx);
    M->hist_cap = t0 + steps;
    DevBuf<double> hist((size_t)std::max<int64_t>(M->hist_cap, 1));
    M->loss_hist = std::move(hist);
    // one step captured once (the sampled rows and Adam's bias correction
    // follow the step counter in device memory), replayed `steps` times
    if (M->graph) {
      cudaGraphExecDestroy(M->graph);
      M->graph = nullptr;
    }
    cudaGraph_t gr = nullptr;
    const bool prof = ctx->profiling;
    ctx->profiling = false;
    LEO_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    try {
      train_step_enqueue(M, seed, lr);
    } catch (...) {
      cudaStreamEndCapture(ctx->stream, &gr);
      if (gr) cudaGraphDestroy(gr);
      ctx->profiling = prof;
      throw;
    }
    LEO_CUDA(cudaStreamEndCapture(ctx->stream, &gr));
    ctx->profiling = prof;
    const cudaError_t e = cudaGraphInstantiate(&M->graph, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) fail(LEO2D_ERR_CUDA, std::string("graph instantiation: ") + cudaGetErrorString(e));
    for (int s = 0; s < steps; ++s) LEO_CUDA(cudaGraphLaunch(M->graph, ctx->stream));
    if (loss_hist && steps > 0) d2h(ctx, loss_hist, M->loss_hist.p + t0, (size_t)steps);
    ctx_check_status(ctx, "MLP training");
  });
}

leo2d_status leo2d_mlp_predict(leo2d_mlp* M, const float* x, int32_t F, int64_t n, float* y) {
  if (!M || !x || !y) return LEO2D_ERR_BAD_ARG;
  leo2d_ctx* ctx = M->ctx;
  return guard(ctx, [&] {
    LEO_REQUIRE(F >= 1 && F <= kIn, "feature count must be 1..64");
    LEO_REQUIRE(n >= 1, "n must be >= 1");
    LEO_CUDA(cudaSetDevice(ctx->device));
    DevBuf<float> src((size_t)n * F);
    DevBuf<__nv_bfloat16> X((size_t)n * kIn);
    DevBuf<float> Y((size_t)n * kOut);
    h2d(ctx, src.p, x, (size_t)n * F);
    launch(ctx, "mlp_pack", [&] {
      k_pack_x<<<grid_for(n * kIn, 256, ctx->sm_count * 8), 256, 0, ctx->stream>>>(n, F, src.p, X.p, nullptr, 0);
    });
    infer_rows(M, X.p, n, Y.p, nullptr);
    d2h(ctx, y, Y.p, (size_t)n * kOut);
    ctx_check_status(ctx, "MLP inference");
  });
}

leo2d_status leo2d_mlp_site_features(leo2d_ctx* ctx, const leo2d_csr* csr, double twist_deg, float* x_out) {
  if (!ctx || !csr || !x_out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = csr->n;
    DevBuf<double> cfg(2 * (size_t)std::max<int64_t>(n, 1));
    csr_shift_configs(ctx, csr, cfg.p);
    DevBuf<float> xf((size_t)std::max<int64_t>(n, 1) * kFeat);
    if (n > 0)
      launch(ctx, "mlp_features", [&] {
        k_features<<<grid_for(n, 256, ctx->sm_count * 8), 256, 0, ctx->stream>>>(n, 0, cfg.p, csr->grid4.p,
                                                                                 (float)twist_deg, nullptr, xf.p);
      });
    d2h(ctx, x_out, xf.p, (size_t)n * kFeat);
    ctx_sync(ctx);
  });
}

leo2d_status leo2d_mlp_site_sum(leo2d_mlp* M, const leo2d_csr* csr, double twist_deg, double* sum_out) {
  if (!M || !csr || !sum_out) return LEO2D_ERR_BAD_ARG;
  leo2d_ctx* ctx = M->ctx;
  return guard(ctx, [&] {
    LEO_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = csr->n;
    LEO_REQUIRE(n >= 1, "empty matrix");
    DevBuf<double> cfg(2 * (size_t)n), sums(kOut);
    csr_shift_configs(ctx, csr, cfg.p);
    DevBuf<__nv_bfloat16> X((size_t)n * kIn);
    launch(ctx, "mlp_features", [&] {
      k_features<<<grid_for(n, 256, ctx->sm_count * 8), 256, 0, ctx->stream>>>(n, 0, cfg.p, csr->grid4.p,
                                                                               (float)twist_deg, X.p, nullptr);
    });
    infer_rows(M, X.p, n, nullptr, sums.p);
    d2h(ctx, sum_out, sums.p, kOut);
    ctx_check_status(ctx, "MLP site sum");
  });
}

// Control-variate trace moments (see leo2d_gpu.h).
leo2d_status leo2d_kpm_dos_cv(leo2d_ctx* ctx, const leo2d_csr* csr, leo2d_mlp* M, const leo2d_kpm_cfg* cfg,
                              double twist_deg, int64_t num_sites, uint64_t site_seed, const double* weights,
                              double* mu_out, double* parts_out) {
  if (!ctx || !csr || !M || !cfg || !mu_out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    const int P = cfg->poly_order;
    LEO_REQUIRE(P >= 4 && P % 4 == 0, "poly_order must be a positive multiple of 4");
    LEO_REQUIRE(num_sites >= 0, "num_sites must be >= 0");
    LEO_REQUIRE(M->ctx == ctx, "the network belongs to another context");
    LEO_REQUIRE(!csr->complex_h, "the control variate is trained on real Hamiltonians (no magnetic field)");
    auto check = [&](leo2d_status st) {
      if (st != LEO2D_OK) fail(st, ctx->last_error);
    };
    LEO_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = csr->n;
    const int Pc = std::min(P, kOut);  // moments covered by the network (even)
    // (1) random-phase estimate of every moment: mean over the vectors
    std::vector<double> phase(P, 0.0);
    const int R = cfg->num_vectors;
    if (R > 0) {
      std::vector<double> mu((size_t)R * P);
      check(leo2d_kpm_dos(ctx, csr, cfg, nullptr, mu.data()));
      for (int v = 0; v < R; ++v)
        for (int j = 0; j < P; ++j) phase[j] += mu[(size_t)v * P + j];
      for (int j = 0; j < P; ++j) phase[j] /= R;
    }
    // (2) the network's sum over every orbital
    std::vector<double> F(kOut, 0.0);
    check(leo2d_mlp_site_sum(M, csr, twist_deg, F.data()));
    // (3) exact moments at uniformly drawn orbitals minus the network there
    std::vector<double> corr(kOut, 0.0);
    if (num_sites > 0) {
      std::vector<int64_t> sites((size_t)num_sites);
      uint64_t st = site_seed;
      for (auto& x : sites) x = (int64_t)(((unsigned __int128)splitmix(st) * (uint64_t)n) >> 64);
      leo2d_kpm_cfg lc = *cfg;
      lc.poly_order = ((Pc + 3) / 4) * 4;
      lc.num_vectors = 1;
      std::vector<double> ld((size_t)num_sites * lc.poly_order);
      check(leo2d_kpm_ldos(ctx, csr, &lc, sites.data(), num_sites, ld.data()));
      DevBuf<int64_t> drows((size_t)num_sites);
      h2d(ctx, drows.p, sites.data(), (size_t)num_sites);
      DevBuf<double> dcfg(2 * (size_t)n);
      csr_shift_configs(ctx, csr, dcfg.p);
      DevBuf<__nv_bfloat16> X((size_t)num_sites * kIn);
      DevBuf<float> Y((size_t)num_sites * kOut);
      launch(ctx, "mlp_features", [&] {
        k_features_at<<<grid_for(num_sites, 256, ctx->sm_count * 8), 256, 0, ctx->stream>>>(
            num_sites, drows.p, dcfg.p, csr->grid4.p, (float)twist_deg, X.p);
      });
      infer_rows(M, X.p, num_sites, Y.p, nullptr);
      std::vector<float> f((size_t)num_sites * kOut);
      d2h(ctx, f.data(), Y.p, f.size());
      ctx_check_status(ctx, "control-variate sites");
      for (int64_t s_ = 0; s_ < num_sites; ++s_)
        for (int j = 0; j < Pc; ++j)
          corr[j] += ld[(size_t)s_ * lc.poly_order + j] - (double)f[(size_t)s_ * kOut + j];
      for (int j = 0; j < Pc; ++j) corr[j] = corr[j] / (double)num_sites * (double)n;
    }
    for (int j = 0; j < P; ++j) {
      if (j < Pc) {
        const double w = weights ? weights[j] : 1.0;
        const double cv = F[j] + corr[j];
        mu_out[j] = w * cv + (1.0 - w) * phase[j];
      } else {
        mu_out[j] = phase[j];
      }
    }
    if (parts_out) {
      for (int j = 0; j < kOut; ++j) {
        parts_out[j] = F[j];
        parts_out[kOut + j] = corr[j];
        parts_out[2 * kOut + j] = j < P ? phase[j] : 0.0;
      }
    }
  });
}

}  // extern "C"
