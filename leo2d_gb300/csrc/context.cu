// context.cu - context life cycle, errors, profiling counters and the
// device-wide scan/reduce used by assembly.
#include <cstring>

#include "common.cuh"

using namespace leo2d;

namespace leo2d {

cudaEvent_t ctx_event(leo2d_ctx* ctx) {
  if (!ctx->free_events.empty()) {
    cudaEvent_t e = ctx->free_events.back();
    ctx->free_events.pop_back();
    return e;
  }
  cudaEvent_t e;
  LEO_CUDA(cudaEventCreate(&e));
  return e;
}

void ctx_sync(leo2d_ctx* ctx) {
  LEO_CUDA(cudaStreamSynchronize(ctx->stream));
  for (auto& t : ctx->pending) {
    float ms = 0.f;
    LEO_CUDA(cudaEventElapsedTime(&ms, t.start, t.stop));
    KStat& s = ctx->stats[t.name];
    s.launches += 1;
    s.ms += ms;
    ctx->free_events.push_back(t.start);
    ctx->free_events.push_back(t.stop);
  }
  ctx->pending.clear();
}

void ctx_check_status(leo2d_ctx* ctx, const char* where) {
  int st = 0;
  LEO_CUDA(cudaMemcpyAsync(&st, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  ctx_sync(ctx);
  if (st == kStatusOk) return;
  LEO_CUDA(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream));
  LEO_CUDA(cudaStreamSynchronize(ctx->stream));
  if (st == kStatusTimeout) fail(LEO2D_ERR_TIMEOUT, std::string(where) + ": device wait ran out");
  if (st == kStatusNonfinite) fail(LEO2D_ERR_NONFINITE, std::string(where) + ": non-finite value");
  fail(LEO2D_ERR_CUDA, std::string(where) + ": device reported an out-of-range index");
}

// ---------------------------------------------------------------- scan

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// Block-level exclusive scan of one tile; writes the tile total to sums[blockIdx].
__global__ void k_scan_tile(const int64_t* __restrict__ in, int64_t* __restrict__ out,
                            int64_t* __restrict__ sums, int64_t n) {
  __shared__ int64_t warp_tot[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t local = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int64_t idx = base + i;
    v[i] = idx < n ? in[idx] : 0;
    local += v[i];
  }
  // inclusive warp scan of per-thread totals
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (unsigned)o) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int64_t t = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= (unsigned)o) t += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = t;  // inclusive over warps
  }
  __syncthreads();
  int64_t run = (warp > 0 ? warp_tot[warp - 1] : 0) + incl - local;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int64_t idx = base + i;
    if (idx < n) out[idx] = run;
    run += v[i];
  }
  if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(int64_t* __restrict__ out, const int64_t* __restrict__ offs, int64_t n) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  const int64_t add = offs[blockIdx.x];
  for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
    int64_t idx = base + i;
    if (idx < n) out[idx] += add;
  }
}

__global__ void k_set_total(int64_t* out, const int64_t* in, int64_t n) {
  // out[n] = out[n-1] + in[n-1]
  out[n] = n > 0 ? out[n - 1] + in[n - 1] : 0;
}

void scan_rec(leo2d_ctx* ctx, const int64_t* in, int64_t* out, int64_t n) {
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  DevBuf<int64_t> sums(tiles + 1), offs(tiles + 1);
  launch(ctx, "scan_tile", [&] {
    k_scan_tile<<<(unsigned)tiles, kScanThreads, 0, ctx->stream>>>(in, out, sums.p, n);
  });
  if (tiles > 1) {
    scan_rec(ctx, sums.p, offs.p, tiles);
    launch(ctx, "scan_add", [&] {
      k_scan_add<<<(unsigned)tiles, kScanThreads, 0, ctx->stream>>>(out, offs.p, n);
    });
  }
  // keep the temporaries alive until the kernels that read them have run
  LEO_CUDA(cudaStreamSynchronize(ctx->stream));
}

__global__ void k_reduce_i64(const int64_t* __restrict__ in, int64_t n, unsigned long long* out) {
  int64_t s = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += in[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, (unsigned long long)s);
}

}  // namespace

void exclusive_scan_i64(leo2d_ctx* ctx, const int64_t* in, int64_t* out, int64_t n) {
  if (n <= 0) {
    LEO_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), ctx->stream));
    return;
  }
  scan_rec(ctx, in, out, n);
  launch(ctx, "scan_total", [&] { k_set_total<<<1, 1, 0, ctx->stream>>>(out, in, n); });
}

int64_t reduce_sum_i64(leo2d_ctx* ctx, const int64_t* in, int64_t n) {
  DevBuf<unsigned long long> acc(1);
  LEO_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(unsigned long long), ctx->stream));
  if (n > 0)
    launch(ctx, "reduce_i64", [&] {
      k_reduce_i64<<<grid_for(n, 256, (int64_t)ctx->sm_count * 8), 256, 0, ctx->stream>>>(in, n, acc.p);
    });
  unsigned long long h = 0;
  d2h(ctx, &h, acc.p, 1);
  ctx_sync(ctx);
  return (int64_t)h;
}

}  // namespace leo2d

// ---------------------------------------------------------------- C ABI

extern "C" {

int leo2d_abi_version(void) { return LEO2D_ABI_VERSION; }

const char* leo2d_status_string(leo2d_status s) {
  switch (s) {
    case LEO2D_OK: return "ok";
    case LEO2D_ERR_BAD_ARG: return "bad argument";
    case LEO2D_ERR_OOM: return "out of memory";
    case LEO2D_ERR_CUDA: return "CUDA error";
    case LEO2D_ERR_TIMEOUT: return "device wait timed out";
    case LEO2D_ERR_NONFINITE: return "non-finite value";
    case LEO2D_ERR_UNSUPPORTED: return "unsupported option";
    case LEO2D_ERR_IO: return "I/O error";
  }
  return "unknown status";
}

leo2d_status leo2d_ctx_create(leo2d_ctx** out, int device) {
  if (!out) return LEO2D_ERR_BAD_ARG;
  *out = nullptr;
  leo2d_ctx* ctx = nullptr;
  try {
    ctx = new leo2d_ctx();
  } catch (...) {
    return LEO2D_ERR_OOM;
  }
  leo2d_status st = guard(ctx, [&] {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
      fail(LEO2D_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    LEO_REQUIRE(device >= 0 && device < count, "device index out of range");
    ctx->device = device;
    LEO_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    LEO_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10)
      fail(LEO2D_ERR_UNSUPPORTED, std::string("this library is built for sm_103a; device is ") + prop.name);
    ctx->sm_count = prop.multiProcessorCount;
    ctx->l2_bytes = prop.l2CacheSize;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    LEO_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->status.alloc(1);
    LEO_CUDA(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream));
    LEO_CUDA(cudaStreamSynchronize(ctx->stream));
  });
  if (st != LEO2D_OK) {
    // keep the message reachable through a process-wide fallback
    static thread_local std::string msg;
    msg = ctx->last_error;
    fprintf(stderr, "leo2d_ctx_create: %s\n", msg.c_str());
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return st;
  }
  *out = ctx;
  return LEO2D_OK;
}

leo2d_status leo2d_ctx_destroy(leo2d_ctx* ctx) {
  if (!ctx) return LEO2D_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& t : ctx->pending) {
    cudaEventDestroy(t.start);
    cudaEventDestroy(t.stop);
  }
  for (auto e : ctx->free_events) cudaEventDestroy(e);
  ctx->status.release();
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return LEO2D_OK;
}

const char* leo2d_last_error(const leo2d_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

void* leo2d_ctx_stream(leo2d_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

leo2d_status leo2d_ctx_set_spin_limit(leo2d_ctx* ctx, uint64_t iterations) {
  if (!ctx) return LEO2D_ERR_BAD_ARG;
  ctx->spin_limit = iterations ? iterations : (1ull << 26);
  return LEO2D_OK;
}

leo2d_status leo2d_ctx_set_profiling(leo2d_ctx* ctx, int enable) {
  if (!ctx) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    ctx_sync(ctx);
    ctx->profiling = enable != 0;
  });
}

leo2d_status leo2d_ctx_kernel_stats(leo2d_ctx* ctx, const char* kernel, int64_t* launches,
                                    double* total_ms) {
  if (!ctx || !kernel) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    ctx_sync(ctx);
    auto it = ctx->stats.find(kernel);
    if (launches) *launches = it == ctx->stats.end() ? 0 : it->second.launches;
    if (total_ms) *total_ms = it == ctx->stats.end() ? 0.0 : it->second.ms;
  });
}

leo2d_status leo2d_ctx_reset_stats(leo2d_ctx* ctx) {
  if (!ctx) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    ctx_sync(ctx);
    ctx->stats.clear();
  });
}

int64_t leo2d_ctx_launch_count(const leo2d_ctx* ctx) { return ctx ? ctx->launches : 0; }

leo2d_status leo2d_ctx_set_option(leo2d_ctx* ctx, const char* key, int64_t value) {
  if (!ctx || !key) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    const std::string k(key);
    if (k == "step_kernel") {
      LEO_REQUIRE(value >= -1 && value <= 5 && value != 4,
                  "step_kernel must be -1 (autotuned), 0 (tiled), 1 (register), 2 (tensor cores), 3 (row blocks) "
                  "or 5 (row blocks of 8 on the tensor cores)");
      ctx->kernel_variant = (int)value;
    } else if (k == "rb_packed") {
      LEO_REQUIRE(value >= -1 && value <= 1, "rb_packed must be -1 (autotuned), 0 or 1");
      ctx->rb_packed = (int)value;
    } else if (k == "rb_warps") {
      LEO_REQUIRE(value == 0 || value == 16 || value == 24 || value == 32, "rb_warps must be 0, 16, 24 or 32");
      ctx->rb_warps = (int)value;
    } else if (k == "rb_window") {
      LEO_REQUIRE(value >= -1 && value <= 1, "rb_window must be -1 (autotuned), 0 or 1");
      ctx->rb_window = (int)value;
    } else if (k == "rt_warps") {
      LEO_REQUIRE(value == 0 || value == 8 || value == 12 || value == 16 || value == 20 || value == 24,
                  "rt_warps must be 0 (autotuned), 8, 12, 16, 20 or 24");
      ctx->rt_warps = (int)value;
    } else if (k == "rt_depth") {
      LEO_REQUIRE(value == 0 || value == 2 || value == 3 || value == 4 || value == 6 || value == 7,
                  "rt_depth must be 0 (autotuned), 2, 3, 4, 6 (rows in registers) or 3, 7 (shared memory)");
      ctx->rt_depth = (int)value;
    } else if (k == "rt_stage") {
      LEO_REQUIRE(value >= -1 && value <= 2,
                  "rt_stage must be -1 (autotuned), 0 (registers), 1 (shared memory by cp.async) or 2 (shared "
                  "memory by TMA gathers)");
      ctx->rt_stage = (int)value;
    } else if (k == "rt_rows") {
      LEO_REQUIRE(value == 0 || value == 8 || value == 16, "rt_rows must be 0 (autotuned), 8 or 16");
      ctx->rt_rows = (int)value;
    } else if (k == "rt_group") {
      LEO_REQUIRE(value >= 0 && value <= 16, "rt_group must be 0 (default) or 1..16");
      ctx->rt_group = (int)value;
    } else if (k == "rt_chunk") {
      LEO_REQUIRE(value >= 0 && value <= 64, "rt_chunk must be 0 (default) or 1..64");
      ctx->rt_chunk = (int)value;
    } else if (k == "alloc_cap_mb") {
      LEO_REQUIRE(value >= 0, "alloc_cap_mb must be >= 0 (0: no limit)");
      ctx->alloc_cap = (size_t)value << 20;
    } else if (k == "mlp_fused") {
      LEO_REQUIRE(value == 0 || value == 1, "mlp_fused must be 0 (one GEMM per layer) or 1 (one fused launch)");
      ctx->mlp_fused = (int)value;
    } else if (k == "reorder_curve") {
      LEO_REQUIRE(value == 0 || value == 1, "reorder_curve must be 0 or 1");
      ctx->reorder_curve = (int)value;
    } else if (k == "rb_unroll") {
      LEO_REQUIRE(value == 0 || value == 4 || value == 8, "rb_unroll must be 0 (autotuned), 4 or 8");
      ctx->rb_unroll = (int)value;
    } else if (k == "test_unsatisfied_wait") {
      // every tiled step waits on an mbarrier that never completes, gives up
      // after the spin limit and reports LEO2D_ERR_TIMEOUT (tests the bounded
      // wait without faulting or hanging anything)
      ctx->test_unsatisfied_wait = value != 0;
    } else if (k == "tile_stages") {
      LEO_REQUIRE(value >= 2 && value <= 4, "tile_stages must be 2..4");
      ctx->tile_stages = (int)value;
    } else if (k == "tile_chunk") {
      LEO_REQUIRE(value >= 1 && value <= 65536, "tile_chunk must be 1..65536");
      ctx->tile_chunk = (int)value;
    } else if (k == "tile_warps") {
      LEO_REQUIRE(value == 0 || value == 8 || value == 24, "tile_warps must be 0, 8 or 24");
      ctx->tile_warps = (int)value;
    } else if (k == "reorder") {
      LEO_REQUIRE(value >= -1 && value <= 1, "reorder must be -1, 0 or 1");
      ctx->reorder = (int)value;
    } else if (k == "kubo_velocity") {
      LEO_REQUIRE(value == -1 || value == 0, "kubo_velocity must be -1 (built in the step) or 0 (stored dxH)");
      ctx->kubo_velocity = (int)value;
    } else if (k == "kubo_chunk") {
      LEO_REQUIRE(value == 0 || (value >= 4 && value % 4 == 0), "kubo_chunk must be 0 or a multiple of 4");
      ctx->kubo_chunk = value;
    } else if (k == "reorder_patch_dA") {
      LEO_REQUIRE(value == 0 || (value >= 5 && value <= 2000),
                  "reorder_patch_dA must be 0 (per step kernel) or 5..2000 (tenths of A)");
      ctx->reorder_patch = value / 10.0;
    } else {
      fail(LEO2D_ERR_BAD_ARG, "unknown option " + k);
    }
  });
}

}  // extern "C"
