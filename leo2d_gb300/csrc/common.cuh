// common.cuh - context, errors, device buffers and launch helpers shared by
// every translation unit of libleo2d_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/leo2d_gpu.h"

namespace leo2d {

struct Error : std::exception {
  leo2d_status status;
  std::string msg;
  Error(leo2d_status s, std::string m) : status(s), msg(std::move(m)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};

[[noreturn]] inline void fail(leo2d_status s, const std::string& m) { throw Error(s, m); }

#define LEO_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      if (e_ == cudaErrorMemoryAllocation)                                              \
        ::leo2d::fail(LEO2D_ERR_OOM, std::string(#call) + ": " + cudaGetErrorString(e_)); \
      ::leo2d::fail(LEO2D_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
    }                                                                                   \
  } while (0)

#define LEO_REQUIRE(cond, msg)                          \
  do {                                                  \
    if (!(cond)) ::leo2d::fail(LEO2D_ERR_BAD_ARG, msg); \
  } while (0)

// Largest single device allocation the calling context allows, in bytes (0: no
// limit): the context's "alloc_cap_mb" option, in force for the duration of one
// API call (guard() sets it for the calling thread).
inline thread_local size_t g_alloc_cap = 0;

// Owning device allocation (move-only).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    if (g_alloc_cap && count * sizeof(T) > g_alloc_cap)
      fail(LEO2D_ERR_OOM, "device allocation of " + std::to_string(count * sizeof(T)) +
                              " bytes exceeds the context's alloc_cap_mb");
    LEO_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};

struct KStat {
  int64_t launches = 0;
  double ms = 0.0;
};

struct PendingTimer {
  std::string name;
  cudaEvent_t start, stop;
};

// Device-side status word written by bounded waits (see kStatus*).
enum : int { kStatusOk = 0, kStatusTimeout = 1, kStatusNonfinite = 2, kStatusBadIndex = 3 };

}  // namespace leo2d

struct leo2d_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  uint64_t spin_limit = 1ull << 26;
  bool profiling = false;
  int sm_count = 0;
  size_t l2_bytes = 0;
  size_t smem_optin = 0;
  std::map<std::string, leo2d::KStat> stats;
  std::vector<leo2d::PendingTimer> pending;
  std::vector<cudaEvent_t> free_events;
  int64_t launches = 0;
  int kernel_variant = -1;    // -1 autotuned, 0 tiled gathers, 1 register gathers, 2 tensor cores, 3 row blocks,
                              // 5 row blocks of 8 on the tensor cores
  int rb_packed = -1;         // row-block step: paired FP32 FMAs (fma.rn.f32x2): -1 autotuned, 0 no, 1 yes
  int rb_warps = 0;           // row-block step: warps per block (= row blocks per tile): 0 autotuned, 16, 24, 32
  int rb_unroll = 0;          // row-block step: slot batches in flight per lane: 0 autotuned, 4, 8
  int rb_window = -1;         // row-block step over shared-memory windows: -1 autotuned, 0 no, 1 yes
  int rt_warps = 0;           // 8-row tensor-core step: warps per CTA: 0 autotuned, 8, 12, 16, 24
  int rt_depth = 0;           // 8-row tensor-core step: k-steps of T_n rows in flight per warp: 0 autotuned,
                              // 2, 3, 4, 6 (rows in registers) or 3, 7 (shared memory)
  int rt_stage = -1;          // 8-row tensor-core step: T_n rows staged in -1 autotuned, 0 registers, 1 shared memory
                              // by cp.async, 2 shared memory by TMA gathers
  int rt_rows = 0;            // tensor-core row-block step: rows per block: 0 autotuned, 8, 16
  int rt_group = 0;           // 8-row tensor-core step: consecutive blocks per warp run: 0 default (2), 1..16
  int rt_chunk = 0;           // 8-row tensor-core step: tiles per CTA between grid-wide jumps: 0 default (2)
  int reorder_curve = 1;      // locality ordering inside a patch: 1 sheet then a fine Hilbert curve, 0 reference index
  int tile_stages = 2;        // shared-memory stages of the tiled kernel
  int test_unsatisfied_wait = 0;  // test hook: tiled steps first wait on a barrier nobody completes
  bool tc_gemm_ready = false;     // shared-memory attributes of the tensor-core GEMM set on this device
  int tile_chunk = 4;         // consecutive tiles per block between grid-wide jumps
  int tile_warps = 0;         // warps per block of the tiled kernel (0 = per shape, 8 or 24)
  int reorder = -1;           // locality ordering: -1 auto, 0 off, 1 on
  double reorder_patch = 0.0;   // patch edge (A); 0: the step kernel's own (16 A; 32 A for row blocks)
  size_t alloc_cap = 0;       // largest single device allocation of a call, bytes (0: no limit)
  int kubo_velocity = -1;     // Kubo trace: -1 D built in the row-block step where possible, 0 stored dxH
  int64_t kubo_chunk = 0;     // Kubo trace: B-side moments held at once (0: as many as memory allows)
  int mlp_fused = 1;          // network forward over many sites: 1 one fused launch, 0 one GEMM per layer
  leo2d::DevBuf<int> status;  // one int, reset before kernels that may set it
};

namespace leo2d {

// Runs f, converting exceptions into a status and the context's last error.
template <class F>
leo2d_status guard(leo2d_ctx* ctx, F&& f) {
  struct CapScope {  // the context's allocation cap for this call, restored on exit
    size_t saved;
    explicit CapScope(size_t cap) : saved(g_alloc_cap) { g_alloc_cap = cap; }
    ~CapScope() { g_alloc_cap = saved; }
  } cap_scope(ctx ? ctx->alloc_cap : g_alloc_cap);
  try {
    f();
    if (ctx) ctx->last_error.clear();
    return LEO2D_OK;
  } catch (const Error& e) {
    if (ctx) ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->last_error = "host allocation failed";
    return LEO2D_ERR_OOM;
  } catch (const std::exception& e) {
    if (ctx) ctx->last_error = e.what();
    return LEO2D_ERR_CUDA;
  } catch (...) {
    if (ctx) ctx->last_error = "unknown error";
    return LEO2D_ERR_CUDA;
  }
}

cudaEvent_t ctx_event(leo2d_ctx* ctx);
// Synchronises the context stream and folds finished timers into the stats.
void ctx_sync(leo2d_ctx* ctx);
// Reads and clears the device status word; throws on a non-zero code.
void ctx_check_status(leo2d_ctx* ctx, const char* where);

// Launches `f` (which enqueues exactly one kernel on ctx->stream), counts it and,
// when profiling is on, brackets it with CUDA events on the same stream.
template <class F>
void launch(leo2d_ctx* ctx, const char* name, F&& f) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (ctx->profiling) {
    a = ctx_event(ctx);
    b = ctx_event(ctx);
    LEO_CUDA(cudaEventRecord(a, ctx->stream));
  }
  f();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) fail(LEO2D_ERR_CUDA, std::string("launch of ") + name + ": " + cudaGetErrorString(e));
  ctx->launches += 1;
  if (ctx->profiling) {
    LEO_CUDA(cudaEventRecord(b, ctx->stream));
    ctx->pending.push_back(PendingTimer{name, a, b});
  } else {
    ctx->stats[name].launches += 1;
  }
}

inline unsigned grid_for(int64_t work, int per_block, int64_t cap = (1ll << 31) - 1) {
  int64_t g = (work + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

template <class T>
void h2d(leo2d_ctx* ctx, T* dst, const T* src, size_t count) {
  if (count) LEO_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
}
template <class T>
void d2h(leo2d_ctx* ctx, T* dst, const T* src, size_t count) {
  if (count) LEO_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
}

// Exclusive prefix sum of n int64 values: out[0..n] with out[n] = total.
// `out` may alias `in` only if it is a distinct buffer of n+1 elements.
void exclusive_scan_i64(leo2d_ctx* ctx, const int64_t* in, int64_t* out, int64_t n);

// Sum of n int64 values (device), returned to the host.
int64_t reduce_sum_i64(leo2d_ctx* ctx, const int64_t* in, int64_t n);

}  // namespace leo2d
