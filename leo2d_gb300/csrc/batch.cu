// batch.cu - many flakes (matrices of uneven size) in one launch per Chebyshev
// step, the whole run captured once in a CUDA graph and replayed.
//
// The reference farms jobs (one flake / twist angle each) to MPI ranks and runs
// Locality::computeDosTraceKPM on each (src/locality.cpp:2295-2309, 6138-6346).
// Here a batch of F flakes shares the GPU inside every step launch:
//   - the grid (SMs x resident blocks) is split into F groups of consecutive
//     blocks (at least one per flake, the rest handed out so that the largest
//     bytes per step per block is as small as it can be); a block runs the
//     step body (tiled CSR, or the row-block step) on its flake's matrix as
//     block `bid` of its group, so its tiles, moment partials and the deferred
//     fixed-order reduction stay within the flake (deterministic);
//   - per-flake arguments travel in one by-value kernel parameter block
//     (__grid_constant__, up to 64 flakes) and all flakes use one shared-memory
//     tile layout (the largest tile of any flake sets its capacity);
//   - one run = for each pass over a block of C columns: per-flake vector fills,
//     P/2 step launches, per-flake final reductions. That sequence is captured
//     into a CUDA graph at creation; a run updates the (seed, first vector) pair
//     in device memory and replays the graph.
// Vector blocks of all flakes are slices of two concatenated n_total x C
// buffers; each flake streams its locality-reordered copy when it has one
// (the same policy as the single-matrix recursion).
#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <vector>

#include "step_kernels.cuh"

using namespace leo2d;

namespace {

constexpr int kMaxFlakes = 64;

template <typename T>
struct BatchParams {
  TileArgs<T> f[kMaxFlakes];
  int block_first[kMaxFlakes + 1];  // flake f owns blocks [block_first[f], block_first[f+1])
  int nflakes;
};

// kernel parameters may take up to 32764 bytes (CUDA 12.1+, sm_70+)
static_assert(sizeof(BatchParams<float>) <= 32764, "batched step parameters exceed the parameter space");

// Row slots of a block of the FP32 tiled step (as the single-matrix kernel).
int batch_slots(int cols, int warps) {
  const int v = cols == 8 ? 2 : 4;
  return warps * (32 / (cols / v));
}

template <typename T, int V, int LPR, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, WARPS == 8 ? 3 : 1)
    k_cheb_batch(const __grid_constant__ BatchParams<T> p) {
  int f = 0;
  while (f + 1 < p.nflakes && (int)blockIdx.x >= p.block_first[f + 1]) ++f;
  tile_body<T, V, LPR, WARPS>(p.f[f], (int)blockIdx.x - p.block_first[f],
                              p.block_first[f + 1] - p.block_first[f]);
}

// Phase columns of one flake from (seed, first vector) in device memory, so a
// captured graph can be replayed with new vectors.
__global__ void k_batch_fill_phase(int64_t n, int C, float* __restrict__ x, const uint64_t* __restrict__ sf,
                                   uint64_t pass_first, int n_complex, const int32_t* __restrict__ new2old) {
  const uint64_t seed = sf[0], first = sf[1] + pass_first;
  const int64_t total = n * C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = new2old ? (int64_t)new2old[e / C] : e / C;
    const int c = (int)(e % C);
    x[e] = (c >> 1) < n_complex ? (float)phase_entry(row, c, seed, first) : 0.0f;
  }
}

template <int C>
__global__ void __launch_bounds__(kThreads) k_batch_reduce(const double* __restrict__ partials,
                                                           double* __restrict__ out, int nb) {
  reduce_prev<C>(partials, out, nb, 0, 1);
}

template <int V, int LPR, int WARPS>
void batch_kernel_w(leo2d_ctx* ctx, unsigned grid, size_t smem, const BatchParams<float>* p, int* occ,
                    size_t set_smem) {
  if (occ) {
    LEO_CUDA(cudaFuncSetAttribute(k_cheb_batch<float, V, LPR, WARPS>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)set_smem));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k_cheb_batch<float, V, LPR, WARPS>, WARPS * 32, set_smem);
    return;
  }
  launch(ctx, "cheb_batch_step",
         [&] { k_cheb_batch<float, V, LPR, WARPS><<<grid, WARPS * 32, smem, ctx->stream>>>(*p); });
}

template <int V, int LPR>
void batch_kernel_t(leo2d_ctx* ctx, unsigned grid, size_t smem, const BatchParams<float>* p, int* occ,
                    size_t set_smem, int warps) {
  if (warps == 24) return batch_kernel_w<V, LPR, 24>(ctx, grid, smem, p, occ, set_smem);
  return batch_kernel_w<V, LPR, 8>(ctx, grid, smem, p, occ, set_smem);
}

void batch_dispatch(leo2d_ctx* ctx, int cols, unsigned grid, size_t smem, const BatchParams<float>* p, int* occ,
                    size_t set_smem, int warps) {
  switch (cols) {
    case 8: return batch_kernel_t<2, 4>(ctx, grid, smem, p, occ, set_smem, warps);
    case 16: return batch_kernel_t<4, 4>(ctx, grid, smem, p, occ, set_smem, warps);
    case 32: return batch_kernel_t<4, 8>(ctx, grid, smem, p, occ, set_smem, warps);
    case 64: return batch_kernel_t<4, 16>(ctx, grid, smem, p, occ, set_smem, warps);
    case 128: return batch_kernel_t<4, 32>(ctx, grid, smem, p, occ, set_smem, warps);
  }
  fail(LEO2D_ERR_BAD_ARG, "batch block width must be 8, 16, 32, 64 or 128 columns");
}

void batch_reduce(leo2d_ctx* ctx, int cols, const double* partials, double* out, int nb) {
  auto go = [&](auto kern) {
    launch(ctx, "batch_reduce", [&] { kern<<<1, kThreads, 0, ctx->stream>>>(partials, out, nb); });
  };
  switch (cols) {
    case 8: return go(k_batch_reduce<8>);
    case 16: return go(k_batch_reduce<16>);
    case 32: return go(k_batch_reduce<32>);
    case 64: return go(k_batch_reduce<64>);
    case 128: return go(k_batch_reduce<128>);
  }
  fail(LEO2D_ERR_BAD_ARG, "unsupported block width");
}

// What a flake streams: its locality-reordered copy when it has one.
struct FlakeView {
  const leo2d_csr* csr = nullptr;
  int64_t n = 0, nnz = 0;
  const int64_t* rowptr = nullptr;
  const uint2* ent = nullptr;
  const int32_t* new2old = nullptr;
  int64_t row_off = 0;  // first row of the flake in the concatenated vector buffers
};

int64_t tile_max_nnz(leo2d_ctx* ctx, const int64_t* rp, int64_t n, int tile_rows) {
  DevBuf<unsigned long long> mx(1);
  LEO_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), ctx->stream));
  const int64_t tiles = (n + tile_rows - 1) / tile_rows;
  launch(ctx, "tile_max_nnz", [&] {
    k_tile_max_nnz<<<grid_for(tiles, 256, (int64_t)ctx->sm_count * 8), 256, 0, ctx->stream>>>(rp, n, tile_rows,
                                                                                            mx.p);
  });
  unsigned long long h = 0;
  d2h(ctx, &h, mx.p, 1);
  ctx_sync(ctx);
  return (int64_t)h;
}

// Shape of the batched step: the tiled CSR step, or the row-block step of
// rb_spmm.cu (32 columns, 24 warps, each flake's locality-ordered row blocks).
struct BatchShape {
  int cols = 32, warps = 8, rows_per_item = 0;
  bool rb = false;
  bool rt = false;  // every step of a pass in one cooperative launch of the 8-row step
};

}  // namespace

struct leo2d_batch {
  leo2d_ctx* ctx = nullptr;
  std::vector<FlakeView> fl;
  int P = 0, steps = 0, R = 0, passes = 0;
  BatchShape shape;
  int tile_rows = 0, tile_cap = 0, rp_bytes = 0, col_bytes = 0, stage_bytes = 0;
  size_t dyn_smem = 0;
  unsigned grid = 0;
  std::vector<int> block_first;
  int64_t n_total = 0;
  DevBuf<float> x0, x1;
  DevBuf<double> partials;  // [2][grid][2C]
  DevBuf<double> dots;      // [passes][F][steps][2C]
  DevBuf<uint64_t> seed_first;
  DevBuf<unsigned> bar;  // 8-row form: per-flake step barriers
  DevBuf<int> abort;
  // 8-row form: what the captured graph points at, per flake (checked before a run)
  std::vector<const unsigned char*> rt_data;
  BatchParams<float> params[2];  // step parity 0 / 1 differ in buffer roles
  cudaGraphExec_t graph = nullptr;
  int64_t launches_per_run = 0;
  ~leo2d_batch() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

namespace {

// Tile layout, grid and flake groups for one shape; returns false if a tile
// of this shape does not fit in shared memory.
bool layout(leo2d_batch* b, const BatchShape& s) {
  leo2d_ctx* ctx = b->ctx;
  const int F = (int)b->fl.size();
  int G = 0;
  std::vector<int64_t> tiles_of(F);
  if (s.rt) {
    b->dyn_smem = rt_batch_smem();
    G = ctx->sm_count;  // one CTA of 16 warps per SM, all resident at once
    // cap[f] below: the chunks of the flake's walk (tile_chunk = 1 in these units)
    for (int f = 0; f < F; ++f) tiles_of[f] = rt_batch_cap(ctx, b->fl[f].csr);
  } else if (s.rb) {
    std::vector<const leo2d_csr*> cs(F);
    for (int f = 0; f < F; ++f) cs[f] = b->fl[f].csr;
    b->dyn_smem = rb_batch_smem(ctx, cs.data(), F, s.warps);
    G = ctx->sm_count;  // one CTA of 24 warps per SM
    for (int f = 0; f < F; ++f) tiles_of[f] = rb_tiles(b->fl[f].csr, s.warps);
  } else {
    const int ns = batch_slots(s.cols, s.warps);
    const int ri = s.rows_per_item > 0 ? s.rows_per_item : std::max(1, 32 / ns);
    b->tile_rows = ns * ri;
    int64_t mx = 0;
    for (auto& f : b->fl) mx = std::max(mx, tile_max_nnz(ctx, f.rowptr, f.n, b->tile_rows));
    auto up = [](int64_t x, int64_t a) { return (x + a - 1) / a * a; };
    b->tile_cap = (int)up(mx + 8, 4);
    b->rp_bytes = (int)up((int64_t)(b->tile_rows + 4) * 8, 128);
    b->col_bytes = (int)up((int64_t)b->tile_cap * 8, 128);
    b->stage_bytes = (int)up(b->rp_bytes + b->col_bytes, 128);
    b->dyn_smem = (size_t)ctx->tile_stages * b->stage_bytes;
    if (b->dyn_smem + 24 * 1024 > ctx->smem_optin) return false;
    int occ = 0;
    batch_dispatch(ctx, s.cols, 0, 0, nullptr, &occ, b->dyn_smem, s.warps);
    G = ctx->sm_count * std::max(occ, 1);
    for (int f = 0; f < F; ++f) tiles_of[f] = (b->fl[f].n + b->tile_rows - 1) / b->tile_rows;
  }
  if (G < F) G = F;
  // blocks per flake: at least one, at most its number of tile chunks, the
  // rest handed out one at a time to the flake whose blocks currently carry
  // the most bytes per step each (the step ends with its slowest block, so this
  // minimises the largest share; proportional rounding left one block with
  // 1.44x the mean work on 32 flakes of 2e4-5e5 orbitals over 152 blocks,
  // this leaves 1.11x)
  std::vector<double> w(F);
  std::vector<int64_t> cap(F);
  for (int f = 0; f < F; ++f) {
    w[f] = (double)b->fl[f].nnz * 8 + (double)b->fl[f].n * (8 + 12.0 * s.cols);
    cap[f] = s.rt ? std::max<int64_t>(1, tiles_of[f])
                  : std::max<int64_t>(1, (tiles_of[f] + ctx->tile_chunk - 1) / ctx->tile_chunk);
  }
  std::vector<int> nb(F, 1);
  {
    auto worse = [&](int x, int y) {  // true if flake y's blocks are more loaded than x's
      const double lx = w[x] / nb[x], ly = w[y] / nb[y];
      return lx < ly || (lx == ly && x > y);
    };
    std::vector<int> heap;
    for (int f = 0; f < F; ++f)
      if (nb[f] < cap[f]) heap.push_back(f);
    std::make_heap(heap.begin(), heap.end(), worse);
    for (int g = F; g < G && !heap.empty(); ++g) {
      std::pop_heap(heap.begin(), heap.end(), worse);
      const int f = heap.back();
      heap.pop_back();
      ++nb[f];
      if (nb[f] < cap[f]) {
        heap.push_back(f);
        std::push_heap(heap.begin(), heap.end(), worse);
      }
    }
  }
  b->block_first.assign(F + 1, 0);
  for (int f = 0; f < F; ++f) b->block_first[f + 1] = b->block_first[f] + nb[f];
  b->grid = (unsigned)b->block_first[F];
  b->shape = s;
  return true;
}

void fill_params(leo2d_batch* b) {
  leo2d_ctx* ctx = b->ctx;
  const int C = b->shape.cols;
  const int F = (int)b->fl.size();
  for (int par = 0; par < 2; ++par) {
    BatchParams<float>& p = b->params[par];
    std::memset(&p, 0, sizeof(p));
    p.nflakes = F;
    for (int f = 0; f <= F; ++f) p.block_first[f] = b->block_first[f];
    for (int f = 0; f < F; ++f) {
      const FlakeView& v = b->fl[f];
      TileArgs<float>& ta = p.f[f];
      StepArgs<float>& a = ta.s;
      a.n = v.n;
      a.rowptr = v.rowptr;
      a.ent = v.ent;
      a.col = nullptr;
      a.val = nullptr;
      a.tn = (par == 0 ? b->x0.p : b->x1.p) + v.row_off * C;
      a.tp = (par == 0 ? b->x1.p : b->x0.p) + v.row_off * C;
      a.alpha = 0.0f;
      a.tprev = nullptr;
      a.rows_per_item = b->shape.rows_per_item;
      ta.lay = TileLayout{ctx->tile_stages, ctx->tile_chunk, b->tile_rows, b->tile_cap, b->rp_bytes, b->col_bytes,
                          b->stage_bytes};
      ta.spin_limit = ctx->spin_limit;
      ta.status = ctx->status.p;
      ta.never_wait = ctx->test_unsatisfied_wait;
    }
  }
}

// One batched step over all flakes: T_{k+1} from T_k (buffer parity k % 2).
void step_launch(leo2d_batch* b, int k, double* partials, const double* prev_partials, const double* dots_pass,
                 bool with_dots) {
  leo2d_ctx* ctx = b->ctx;
  const int C = b->shape.cols, F = (int)b->fl.size(), S = b->steps;
  if (b->shape.rb) {
    std::vector<RbBatchFlake> fl(F);
    for (int f = 0; f < F; ++f) {
      const FlakeView& v = b->fl[f];
      const size_t off = (size_t)b->block_first[f] * 2 * C;
      fl[f].csr = v.csr;
      fl[f].tn = (k % 2 == 0 ? b->x0.p : b->x1.p) + v.row_off * C;
      fl[f].tp = (k % 2 == 0 ? b->x1.p : b->x0.p) + v.row_off * C;
      fl[f].first = k == 0;
      fl[f].partials = partials + off;
      fl[f].prev_partials = prev_partials ? prev_partials + off : nullptr;
      fl[f].prev_dots =
          with_dots && k > 0 ? const_cast<double*>(dots_pass) + ((size_t)f * S + (k - 1)) * 2 * C : nullptr;
    }
    rb_batch_launch(ctx, fl.data(), b->block_first.data(), F, b->shape.warps, b->dyn_smem);
    return;
  }
  BatchParams<float>& p = b->params[k % 2];
  for (int f = 0; f < F; ++f) {
    StepArgs<float>& a = p.f[f].s;
    const size_t off = (size_t)b->block_first[f] * 2 * C;
    a.first = k == 0;
    a.partials = partials + off;
    a.prev_partials = prev_partials ? prev_partials + off : nullptr;
    a.prev_dots =
        with_dots && k > 0 ? const_cast<double*>(dots_pass) + ((size_t)f * S + (k - 1)) * 2 * C : nullptr;
  }
  batch_dispatch(ctx, C, b->grid, b->dyn_smem, &p, nullptr, 0, b->shape.warps);
}

// Enqueues one full run (all passes) on the context stream.
void enqueue_run(leo2d_batch* b) {
  leo2d_ctx* ctx = b->ctx;
  const int C = b->shape.cols, F = (int)b->fl.size(), S = b->steps;
  const int per_pass = C / 2;
  const size_t part = (size_t)b->grid * 2 * C;
  for (int pass = 0; pass < b->passes; ++pass) {
    const int nv = std::min(per_pass, b->R - pass * per_pass);
    for (int f = 0; f < F; ++f) {
      const FlakeView& v = b->fl[f];
      float* x = b->x0.p + v.row_off * C;
      launch(ctx, "batch_fill", [&] {
        k_batch_fill_phase<<<grid_for(v.n * C, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
            v.n, C, x, b->seed_first.p, (uint64_t)pass * per_pass, nv, v.new2old);
      });
    }
    double* dots = b->dots.p + (size_t)pass * F * S * 2 * C;
    if (b->shape.rt) {
      // the pass's S steps in one cooperative launch
      std::vector<RtBatchFlake> fl(F);
      for (int f = 0; f < F; ++f) {
        const FlakeView& v = b->fl[f];
        const leo2d_csr* m = v.csr;
        RtBatchFlake& r = fl[f];
        r.data = m->rt_data.p;
        r.wbeg = m->rt_wbeg.p;
        r.kst = m->rt_kst.p;
        r.n = m->n;
        r.nrb = m->rt_blocks;
        r.group = m->rt_group;
        r.chunk = m->rt_chunk;
        r.x0 = b->x0.p + v.row_off * C;
        r.x1 = b->x1.p + v.row_off * C;
        r.partials[0] = b->partials.p + (size_t)b->block_first[f] * 2 * C;
        r.partials[1] = b->partials.p + part + (size_t)b->block_first[f] * 2 * C;
        r.dots = dots + (size_t)f * S * 2 * C;
      }
      rt_batch_launch(ctx, fl.data(), b->block_first.data(), F, S, b->bar.p, b->abort.p,
                      ctx->test_unsatisfied_wait);
    } else {
      for (int k = 0; k < S; ++k)
        step_launch(b, k, b->partials.p + (size_t)(k % 2) * part,
                    k == 0 ? nullptr : b->partials.p + (size_t)((k + 1) % 2) * part, dots, true);
    }
    for (int f = 0; f < F; ++f) {
      const size_t off = (size_t)b->block_first[f] * 2 * C;
      batch_reduce(ctx, C, b->partials.p + (size_t)((S - 1) % 2) * part + off,
                   dots + ((size_t)f * S + (S - 1)) * 2 * C, b->block_first[f + 1] - b->block_first[f]);
    }
  }
}

// The 8-row form: each flake's blocks built for the CTAs it gets (a single run on
// the same matrix rebuilds them for one CTA per SM, so a run checks them first).
void build_rt_formats(leo2d_batch* b) {
  leo2d_ctx* ctx = b->ctx;
  rt_batch_prepare(ctx, b->grid);
  b->rt_data.assign(b->fl.size(), nullptr);
  for (size_t f = 0; f < b->fl.size(); ++f) {
    leo2d_csr* m = const_cast<leo2d_csr*>(b->fl[f].csr);
    const int nb = b->block_first[f + 1] - b->block_first[f];
    LEO_REQUIRE(csr_build_rt(ctx, m, kRtBatchWarps, rt_group_of(ctx), rt_chunk_of(ctx), 8, nb) &&
                    m->rt_grid == (unsigned)nb,
                "a batched flake's 8-row blocks exceed the build limits");
    b->rt_data[f] = m->rt_data.p;
  }
}

bool rt_formats_current(const leo2d_batch* b) {
  for (size_t f = 0; f < b->fl.size(); ++f) {
    const leo2d_csr* m = b->fl[f].csr;
    const int nb = b->block_first[f + 1] - b->block_first[f];
    if (!m->rt_built || m->rt_data.p != b->rt_data[f] || m->rt_grid != (unsigned)nb || m->rt_rows != 8 ||
        m->rt_warps != kRtBatchWarps)
      return false;
  }
  return true;
}

void allocate(leo2d_batch* b) {
  const int C = b->shape.cols, F = (int)b->fl.size();
  b->bar.alloc((size_t)F);
  b->abort.alloc(1);
  b->x0.alloc((size_t)b->n_total * C);
  b->x1.alloc((size_t)b->n_total * C);
  b->partials.alloc((size_t)2 * b->grid * 2 * C);
  b->passes = (2 * b->R + C - 1) / C;
  b->dots.alloc((size_t)b->passes * F * b->steps * 2 * C);
}

void capture(leo2d_batch* b) {
  leo2d_ctx* ctx = b->ctx;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  const int64_t l0 = ctx->launches;
  const bool prof = ctx->profiling;
  ctx->profiling = false;  // no timing events inside the graph
  cudaGraph_t g = nullptr;
  LEO_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  try {
    enqueue_run(b);
  } catch (...) {
    cudaStreamEndCapture(ctx->stream, &g);
    if (g) cudaGraphDestroy(g);
    ctx->profiling = prof;
    throw;
  }
  LEO_CUDA(cudaStreamEndCapture(ctx->stream, &g));
  ctx->profiling = prof;
  const cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) fail(LEO2D_ERR_CUDA, std::string("graph instantiation: ") + cudaGetErrorString(e));
  b->launches_per_run = ctx->launches - l0;
}

// Times `reps` step launches of the current shape (CUDA events, untimed warm-up).
float time_steps(leo2d_batch* b, int reps) {
  leo2d_ctx* ctx = b->ctx;
  const int C = b->shape.cols, F = (int)b->fl.size();
  const size_t part = (size_t)b->grid * 2 * C;
  for (int f = 0; f < F; ++f) {
    const FlakeView& v = b->fl[f];
    launch(ctx, "batch_fill", [&] {
      k_batch_fill_phase<<<grid_for(v.n * C, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
          v.n, C, b->x0.p + v.row_off * C, b->seed_first.p, 0, C / 2, v.new2old);
    });
  }
  cudaEvent_t e0 = ctx_event(ctx), e1 = ctx_event(ctx);
  for (int k = 0; k < reps + 1; ++k) {
    if (k == 1) LEO_CUDA(cudaEventRecord(e0, ctx->stream));
    step_launch(b, k, b->partials.p + (size_t)(k % 2) * part, nullptr, nullptr, false);
  }
  LEO_CUDA(cudaEventRecord(e1, ctx->stream));
  LEO_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  LEO_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  ctx->free_events.push_back(e0);
  ctx->free_events.push_back(e1);
  ctx_check_status(ctx, "batched Chebyshev step");
  return ms / reps;
}

}  // namespace

extern "C" {

leo2d_status leo2d_batch_create(leo2d_ctx* ctx, const leo2d_csr* const* csrs, int32_t num,
                                const leo2d_kpm_cfg* cfg, leo2d_batch** out) {
  if (!ctx || !csrs || !cfg || !out) return LEO2D_ERR_BAD_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    LEO_REQUIRE(num >= 1 && num <= kMaxFlakes, "a batch holds 1..64 matrices");
    LEO_REQUIRE(cfg->poly_order >= 4 && cfg->poly_order % 4 == 0, "poly_order must be a positive multiple of 4");
    LEO_REQUIRE(cfg->num_vectors >= 1, "num_vectors must be >= 1");
    LEO_REQUIRE(cfg->vector_kind == LEO2D_VEC_PHASE, "batched runs take random-phase vectors");
    LEO_REQUIRE(cfg->precision == LEO2D_FP32, "batched runs use the FP32 recursion (FP64 moments)");
    LEO_REQUIRE(cfg->block == 0 || cfg->block == 8 || cfg->block == 16 || cfg->block == 32 || cfg->block == 64 ||
                    cfg->block == 128,
                "block must be 0 (autotuned), 8, 16, 32, 64 or 128");
    for (int32_t f = 0; f < num; ++f)
      LEO_REQUIRE(csrs[f] && !csrs[f]->complex_h, "batched runs take real Hamiltonians (no magnetic field)");
    LEO_CUDA(cudaSetDevice(ctx->device));
    auto b = std::make_unique<leo2d_batch>();
    b->ctx = ctx;
    b->P = cfg->poly_order;
    b->steps = cfg->poly_order / 2;
    b->R = cfg->num_vectors;
    int64_t off = 0;
    bool rb_mode = (cfg->block == 0 || cfg->block == 32) && ctx->reorder != 0 && ctx->kernel_variant != 0 &&
                   ctx->kernel_variant != 1;
    for (int f = 0; f < num; ++f)
      rb_mode = rb_mode && csrs[f] && csrs[f]->pos.p != nullptr && csrs[f]->nnz > 0;
    for (int f = 0; f < num; ++f) {
      const leo2d_csr* m = csrs[f];
      LEO_REQUIRE(m != nullptr && m->n > 0, "batch matrix is null or empty");
      for (int g = 0; g < f; ++g) LEO_REQUIRE(csrs[g] != m, "a matrix appears twice in the batch");
      leo2d_csr* mm = const_cast<leo2d_csr*>(m);
      LEO_REQUIRE(m->ent.p != nullptr || m->nnz == 0, "matrix has no FP32 values");
      // the row-block step (every flake ordered, 32 columns) unless the tiled step is asked for
      const bool perm = rb_mode || (m->pos.p != nullptr && m->nnz > 0 &&
                                    (ctx->reorder == 1 || (ctx->reorder == -1 && m->n >= 100000)));
      const double patch = reorder_patch_for(ctx, rb_mode);
      if (perm && (!m->reordered || m->reorder_patch != patch || m->reorder_curve_req != ctx->reorder_curve))
        csr_build_reordered(ctx, mm, patch, m->reorder_fp64, ctx->reorder_curve != 0);
      if (rb_mode && ctx->kernel_variant == 3 && (!m->rb_built || m->rb_patch != m->reorder_patch))
        LEO_REQUIRE(csr_build_rb(ctx, mm), "a batched flake's row blocks exceed the build limits");
      FlakeView v;
      v.csr = m;
      v.n = m->n;
      v.nnz = m->nnz;
      v.rowptr = perm ? m->prow.p : m->rowptr.p;
      v.ent = perm ? m->pent.p : m->ent.p;
      v.new2old = perm ? m->new2old.p : nullptr;
      v.row_off = off;
      off += (m->n + 3) / 4 * 4;  // 16-byte aligned slices for any C
      b->fl.push_back(v);
    }
    b->n_total = off;
    b->seed_first.alloc(2);
    uint64_t sf[2] = {cfg->seed, cfg->first_vector};
    h2d(ctx, b->seed_first.p, sf, 2);

    // shape: the caller's, or the fastest estimated run time over widths,
    // warps and rows per slot (each candidate timed on real batched steps)
    std::vector<BatchShape> cands;
    // 32-column passes over ordered flakes: every step of a pass in one launch of
    // the 8-row tensor-core step, or (step_kernel 3) one launch per step of the
    // 4-row step
    if (rb_mode && ctx->kernel_variant == 3) cands.push_back(BatchShape{32, 24, 0, true, false});
    else if (rb_mode) cands.push_back(BatchShape{32, kRtBatchWarps, 0, false, true});
    const int widths[5] = {8, 16, 32, 64, 128};
    for (int w : rb_mode ? std::vector<int>() : std::vector<int>(widths, widths + 5)) {
      if (cfg->block && w != cfg->block) continue;
      if (!cfg->block && w > 2 * ((2 * b->R + 7) / 8 * 4)) continue;  // wider than the vectors need
      for (int warps : {8, 24})
        for (int ri : {0, 2}) {
          if (cfg->rows_per_warp && ri != cfg->rows_per_warp) continue;
          cands.push_back(BatchShape{w, warps, cfg->rows_per_warp ? cfg->rows_per_warp : ri});
        }
    }
    if (cands.empty()) cands.push_back(BatchShape{cfg->block ? cfg->block : 32, 8, cfg->rows_per_warp, false});
    BatchShape best;
    double best_t = 1e300;
    if (cands.size() == 1) {
      LEO_REQUIRE(layout(b.get(), cands[0]), "batch tiles do not fit in shared memory");
      best = cands[0];
    } else {
      for (const auto& s : cands) {
        if (!layout(b.get(), s)) continue;
        allocate(b.get());
        fill_params(b.get());
        const double t_step = time_steps(b.get(), 3);
        const double t_run = t_step * b->steps * ((2 * b->R + s.cols - 1) / s.cols);
        if (t_run < best_t) {
          best_t = t_run;
          best = s;
        }
      }
      LEO_REQUIRE(best_t < 1e300, "batch tiles do not fit in shared memory");
      layout(b.get(), best);
    }
    allocate(b.get());
    fill_params(b.get());
    if (b->shape.rt) build_rt_formats(b.get());
    capture(b.get());
    *out = b.release();
  });
}

leo2d_status leo2d_batch_run(leo2d_batch* b, uint64_t seed, uint64_t first_vector, double* mu_out) {
  if (!b || !mu_out) return LEO2D_ERR_BAD_ARG;
  leo2d_ctx* ctx = b->ctx;
  return guard(ctx, [&] {
    LEO_CUDA(cudaSetDevice(ctx->device));
    if (b->shape.rt && !rt_formats_current(b)) {
      // a single run on one of the flakes rebuilt its blocks for another grid:
      // rebuild them for the batch and capture the run again
      build_rt_formats(b);
      capture(b);
    }
    uint64_t sf[2] = {seed, first_vector};
    h2d(ctx, b->seed_first.p, sf, 2);
    LEO_CUDA(cudaGraphLaunch(b->graph, ctx->stream));
    ctx->launches += b->launches_per_run;
    const int C = b->shape.cols, F = (int)b->fl.size(), S = b->steps;
    std::vector<double> dots((size_t)b->passes * F * S * 2 * C);
    d2h(ctx, dots.data(), b->dots.p, dots.size());
    ctx_check_status(ctx, "batched Chebyshev recursion");
    const int per_pass = C / 2;
    std::vector<double> one((size_t)S * 2 * C);
    for (int f = 0; f < F; ++f)
      for (int pass = 0; pass < b->passes; ++pass) {
        const int nv = std::min(per_pass, b->R - pass * per_pass);
        const double* src = dots.data() + ((size_t)pass * F + f) * S * 2 * C;
        one.assign(src, src + (size_t)S * 2 * C);
        dots_to_moments(one, C, S, 2, nv, mu_out + ((size_t)f * b->R + (size_t)pass * per_pass) * b->P, b->P);
      }
  });
}

leo2d_status leo2d_batch_info(const leo2d_batch* b, int32_t* block_cols, int32_t* warps, int32_t* rows_per_item,
                              int32_t* grid, int64_t* launches_per_run) {
  if (!b) return LEO2D_ERR_BAD_ARG;
  if (block_cols) *block_cols = b->shape.cols;
  if (warps) *warps = b->shape.warps;
  if (rows_per_item) *rows_per_item = b->shape.rows_per_item;
  if (grid) *grid = (int32_t)b->grid;
  if (launches_per_run) *launches_per_run = b->launches_per_run;
  return LEO2D_OK;
}

leo2d_status leo2d_batch_destroy(leo2d_batch* b) {
  if (!b) return LEO2D_OK;
  cudaSetDevice(b->ctx->device);
  delete b;
  return LEO2D_OK;
}

}  // extern "C"
