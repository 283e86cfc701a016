// kpm.cuh - the fused Chebyshev-step SpMM and its drivers, shared by the DOS,
// LDOS, batched and conductivity entry points.
#pragma once

#include "csr.cuh"

namespace leo2d {

// One launch configuration of the step kernel.
struct StepShape {
  int cols = 32;           // real columns per vector block (C)
  int rows_per_item = 0;   // rows per row slot per work item / tile (0 = default)
  bool fp64 = false;
  bool tiled = true;       // bulk-copy tiled kernel (else the register-streaming kernel)
  int warps = 8;           // warps per block of the tiled kernel (8 or 24)
  bool tc = false;         // tensor-core step (tc_spmm.cu) over the locality-ordered tiles
  bool rb = false;         // row-block step (rb_spmm.cu) over the locality-ordered copy (FP32, 32 columns)
  int rb_warps = 24;       // row-block step: warps per block = row blocks per tile (16, 24, 32)
  bool rb_packed = true;   // row-block step: paired FP32 FMAs
  int rb_unroll = 8;       // row-block step: slot batches in flight per lane (4, 8)
  bool rb_window = false;  // row-block step over shared-memory windows (rbw_spmm.cu)
  bool rt = false;         // 8-row blocks on the tensor cores (rt_spmm.cu; FP32, 32 columns)
  int rt_warps = 16;       // 8-row step: warps per CTA (8, 12, 16, 24)
  int rt_depth = 3;        // 8-row step: k-steps of T_n rows in flight per warp (registers 2, 3, 4, 6;
                           // cp.async 3, 7; TMA 3, 7)
  int rt_stage = 1;        // 8-row step: T_n rows staged in 0 registers, 1 shared memory by cp.async,
                           // 2 shared memory by TMA gathers
  int rt_rows = 8;         // rows per block (8; 16 with rt_stage 1)
};

// Vector block resident on the device: two buffers of n x cols (T_k, T_{k-1}).
struct Recursion {
  leo2d_ctx* ctx = nullptr;
  const leo2d_csr* csr = nullptr;
  StepShape shape;
  int64_t n = 0;
  unsigned grid = 0;
  DevBuf<char> x0, x1;          // T buffers (float or double)
  DevBuf<double> partials;      // [grid][cols][2]
  DevBuf<unsigned> counter;     // last-block ticket
  DevBuf<double> dots;          // [steps][cols][2]: <T_k|T_k>, <T_{k+1}|T_k>
  int steps = 0;
  int tile_stages = 2, tile_chunk = 1, tile_rows = 0, tile_cap = 0, tile_rp_bytes = 0, tile_col_bytes = 0, tile_stage_bytes = 0;
  size_t dyn_smem = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = -1;
  bool use_perm = false;  // stream the locality-ordered copy of the matrix
  bool allow_perm = true; // set false before setup() to keep the reference row order
  // the direct moments of a non-Hermitian H~: before step k, direct[k][c] =
  // sum_i T_k[i][c] start[i][c] (FP64), start = a copy of T_0 (FP32 only)
  const float* start = nullptr;
  double* direct = nullptr;
  const int32_t* perm() const { return use_perm ? csr->new2old.p : nullptr; }
  // complex H: vector v occupies columns 2v (real part) and 2v + 1 (imaginary part)
  int pairs() const { return csr->complex_h ? 1 : 0; }

  void setup(leo2d_ctx* c, const leo2d_csr* m, StepShape s, int steps_);
  void* buf(int i) { return i == 0 ? (void*)x0.p : (void*)x1.p; }
  // Enqueues steps [0, steps) on T_0 already in x0; dots land in `dots`.
  void run();
  // Enqueues one step out = alpha M in - prev (no subtraction when first);
  // M = H~ (matrix 0) or dxH (matrix 1); prev may equal out. Block dots unused.
  void step(const void* in, void* out, const void* prev, bool first, double alpha, int matrix);
  ~Recursion();
};

// The tensor-core step (tc_spmm.cu): dynamic shared memory for a block width,
// and one launch (partials / prev_* as in the gather kernels).
size_t tc_smem_bytes(const leo2d_csr* csr, int cols);
void tc_launch_step(leo2d_ctx* ctx, const leo2d_csr* csr, int cols, unsigned grid, size_t smem, const float* tn,
                    float* tp, const float* tprev, int first, float alpha, double* partials,
                    const double* prev_partials, double* prev_dots);

// The row-block step (rb_spmm.cu): shared-memory stages that fit (0: none),
// dynamic shared memory, grid, and one launch.
// (velocity: the stages of the velocity step, which also copy the slots' positions)
int rb_stages(leo2d_ctx* ctx, leo2d_csr* csr, int warps, bool velocity = false);
size_t rb_smem_bytes(leo2d_ctx* ctx, leo2d_csr* csr, int warps, bool velocity = false);
unsigned rb_grid(leo2d_ctx* ctx, const leo2d_csr* csr, int warps);
// With out2 (the velocity step; csr_build_rb_xs first, smem and grid for
// velocity stages) the launch also writes out2 = D T_n, D_ij = (x_i - x_j) H~_ij
// (a flake's dxH), from the same gathers, and computes no moment dots.
void rb_launch_step(leo2d_ctx* ctx, const leo2d_csr* csr, const StepShape& shape, unsigned grid, size_t smem,
                    const float* tn, float* tp, const float* tprev, int first, float alpha, double* partials,
                    const double* prev_partials, double* prev_dots, float* out2 = nullptr);

// The 8-row tensor-core step (rt_spmm.cu): shared memory of a shape, the grid
// its blocks are built for (csr_build_rt with rt_group_of / rt_chunk_of), and
// one launch.
size_t rt_smem_bytes(int warps, int depth, int stage, int rows);
unsigned rt_grid(leo2d_ctx* ctx, const leo2d_csr* csr, int warps, int rows);
int rt_group_of(const leo2d_ctx* ctx);
int rt_chunk_of(const leo2d_ctx* ctx);
void rt_launch_step(leo2d_ctx* ctx, const leo2d_csr* csr, const StepShape& shape, unsigned grid, size_t smem,
                    const float* tn, float* tp, const float* tprev, int first, float alpha, double* partials,
                    const double* prev_partials, double* prev_dots);

// Every step of one pass over several matrices (flakes) in one cooperative
// launch of the 8-row tensor-core step (rt_spmm.cu): flake f runs on CTAs
// [block_first[f], block_first[f+1]), whose count its blocks were built for
// (csr_build_rt's max_grid), and its CTAs meet at a barrier between steps.
constexpr int kRtBatchMax = 64;
constexpr int kRtBatchWarps = 16, kRtBatchDepth = 3;  // the launch shape of every flake
struct RtBatchFlake {
  const unsigned char* data = nullptr;  // the flake's k-steps (csr->rt_data)
  const int64_t* wbeg = nullptr;
  const int64_t* kst = nullptr;
  int64_t n = 0, nrb = 0;
  int group = 0, chunk = 0;
  float* x0 = nullptr;            // T_0 (step parity 0 reads x0, writes x1)
  float* x1 = nullptr;
  double* partials[2] = {nullptr, nullptr};  // by step parity, [CTAs of the flake][64]
  double* dots = nullptr;         // [steps][64] of this pass
};
// CTAs the flake's 8-row blocks can keep busy (its walk's chunks, at most one per SM)
unsigned rt_batch_cap(leo2d_ctx* ctx, const leo2d_csr* csr);
size_t rt_batch_smem();
// Sets the launch's shared-memory attribute and checks that `grid` CTAs can all
// be resident (call outside stream capture, before the first launch).
void rt_batch_prepare(leo2d_ctx* ctx, unsigned grid);
// One launch of `steps` steps over every flake; bar [nflakes] and abort are zeroed
// first (on the stream). never_arrive: the barriers wait for one arrival too many
// (tests the bounded wait).
void rt_batch_launch(leo2d_ctx* ctx, const RtBatchFlake* fl, const int* block_first, int nflakes, int steps,
                     unsigned* bar, int* abort, int never_arrive);

// The row-block step over several matrices (flakes) in one launch: flake f runs
// on CTAs [block_first[f], block_first[f+1]) with its own vectors and partials.
constexpr int kRbBatchMax = 64;
struct RbBatchFlake {
  const leo2d_csr* csr = nullptr;
  const float* tn = nullptr;
  float* tp = nullptr;
  double* partials = nullptr;
  const double* prev_partials = nullptr;
  double* prev_dots = nullptr;
  int first = 0;
};
// shared memory of the widest flake's stages; the tiles of a matrix (chunk units)
size_t rb_batch_smem(leo2d_ctx* ctx, const leo2d_csr* const* csrs, int n, int warps);
int64_t rb_tiles(const leo2d_csr* csr, int warps);
void rb_batch_launch(leo2d_ctx* ctx, const RbBatchFlake* fl, const int* block_first, int nflakes, int warps,
                     size_t smem);

// The windowed row-block step (rbw_spmm.cu), as above.
int rbw_stages(leo2d_ctx* ctx, leo2d_csr* csr);
size_t rbw_smem_bytes(leo2d_ctx* ctx, leo2d_csr* csr);
unsigned rbw_grid(leo2d_ctx* ctx, const leo2d_csr* csr);
void rbw_launch_step(leo2d_ctx* ctx, const leo2d_csr* csr, const StepShape& shape, unsigned grid, size_t smem,
                     const float* tn, float* tp, const float* tprev, int first, float alpha, double* partials,
                     const double* prev_partials, double* prev_dots);

// Patch edge (A) of the locality ordering for a step kernel: the context's
// setting, else 32 A for the row-block step (larger blocks of neighbours, fewer
// slots) and 16 A for the gather kernels (smaller gathered working set).
inline double reorder_patch_for(const leo2d_ctx* ctx, bool row_blocks) {
  return ctx->reorder_patch > 0.0 ? ctx->reorder_patch : (row_blocks ? 32.0 : 16.0);
}

// Chooses the shape for a matrix; cached per context and matrix.
StepShape choose_shape(leo2d_ctx* ctx, const leo2d_csr* csr, bool fp64, int cols_needed,
                       int requested_cols, int requested_rows);

// Fills x0 with the start vectors of one block.
void fill_phase(leo2d_ctx* ctx, Recursion& r, uint64_t seed, uint64_t first_complex, int n_complex);
void fill_gaussian(leo2d_ctx* ctx, Recursion& r, uint64_t seed, uint64_t first_vec, int n_vec);
void fill_host(leo2d_ctx* ctx, Recursion& r, const double* host_vectors, int first_vec, int n_vec);
void fill_unit(leo2d_ctx* ctx, Recursion& r, const int64_t* targets, int n_targets);

// Converts per-column dots of a finished recursion into moments:
// mu[v][2k] = 2 D0_k - mu_0, mu[v][2k+1] = 2 D1_k - mu_1 (mu_0 = D0_0, mu_1 = D1_0),
// with D the sum over the `group` columns of vector v (2 for complex vectors).
void dots_to_moments(const std::vector<double>& dots, int cols, int steps, int group, int n_vec,
                     double* mu_out, int P);

}  // namespace leo2d
