// rt_spmm.cu - the Chebyshev step over row blocks of 8 rows on the tensor cores
// (FP32 recursion, 32 columns).
//
// Same step as the other step kernels (T_{n+1} = a H~ T_n - T_{n-1} with the
// two moment dots fused; Locality::computeDosTraceKPM, src/locality.cpp:
// 6195-6234, with SpMatrix::vectorMultiply, src/matrix/spmatrix.cpp:346-360, as
// its product). The 4-row block step (rb_spmm.cu) is bound by the L1 / shared
// memory pipe: every slot costs one wavefront for the gathered T_n row and one
// for the broadcast of its 4 values. Here 8 consecutive rows (a compact cluster
// of one sheet under the curve ordering of reorder.cu) share the union of their
// columns, and the product of a k-step (8 slots) is two TF32 MMAs per split
// term: D^T (32 columns x 8 rows) = X^T (32 x 8 slots) V^T (8 slots x 8 rows),
// m16n8k8, the 32 columns as M. The tensor core consumes the value panel and
// the staged T_n rows from shared memory at full width, so a slot costs about
// half the pipe work of the 4-row step and 8 rows share each gathered row.
//
// FP32 accuracy from TF32 units: every operand x is split x = hi + lo (hi =
// x rounded to TF32, lo = the rest rounded to TF32) and the product is taken as
// lo*hi + hi*lo + hi*hi, accumulated in FP32 (relative error about 2^-21).
//
// Format (built once per matrix and launch shape, from the locality-ordered copy)
//   row block b = rows 8b..8b+7 of the ordered numbering; its slots are the
//   sorted union of its rows' columns, padded to a multiple of 8 (padding: a
//   valid column with zero values). Slots go in k-steps of 8; a k-step is
//   288 bytes:
//     int32 col[8]       slots in the order 0 4 1 5 2 6 3 7, so lane q of a
//                        quarter-warp reads (slot q, slot q + 4) as one int2
//     float2 v[32]       lane 4g + t holds (V[row g][slot t], V[row g][slot t+4]),
//                        the B fragment of mma.m16n8k8 (B = V^T, k = slot, n = row)
//   Blocks are stored in the order the kernel processes them: warp w of CTA c
//   takes runs of G consecutive blocks (one run per tile of W runs, tiles in
//   chunked round-robin over the CTAs), so each warp streams one contiguous
//   range of k-steps, rt_wbeg[c W + w] .. rt_wbeg[c W + w + 1]; rt_kst holds
//   each block's k-step count (the kernel's block boundaries).
// Kernel (one CTA per SM, W warps, no CTA-wide barrier in the main loop)
//   Each warp runs a software pipeline over its k-steps with cp.async groups:
//   at iteration u it copies the matrix data of k-step u + D + DM and the 8 T_n
//   rows of k-step u + D (the columns come from the matrix data that landed DM
//   iterations earlier), both with cp.async.cg (from L2: keeping the rows in L1
//   for neighbouring blocks hit 46 % but cost an L1 tag wavefront per copy on
//   the pipe that bounds the kernel; 0.68 -> 0.65 ms on a 2.4M-orbital flake),
//   then waits for k-step u's group and runs its MMAs. T_n rows land in a 1 KB ring entry with 16-byte chunk c of row s at
//   chunk c ^ s; lane (g, t) reads columns 4 cg .. 4 cg + 3, cg = (g >> 1) |
//   ((g & 1) << 2), of slots t and t + 4 with no bank conflicts (memory column
//   4 cg + i is logical column g + 8 i of the MMA). At a block's last k-step
//   the lane owns rows 2t and 2t + 1 of the block, columns 4 cg .. 4 cg + 3: it
//   writes T_{n+1} and adds its moment dots (FP32 over 16 blocks, then FP64).
//   cp.async waits are hardware waits on copies already issued: no spin loop.
#include <algorithm>
#include <cmath>
#include <vector>

#include "kpm.cuh"
#include "tc_gemm.cuh"

using namespace leo2d;

#include "step_kernels.cuh"

namespace {

#include "rb_common.cuh"

constexpr int kRtRows = 8;           // rows of an n-tile (and of the 8-row blocks)
constexpr int kRtStepBytes = 288;    // one k-step of an 8-row block: 8 columns + 32 value pairs
// one k-step of a block of R rows: 8 columns + 8 R values
__host__ __device__ constexpr int rt_step_bytes(int R) { return 32 + 32 * R; }
constexpr int kRtMaxEnt = 2048;      // stored entries of one block (build limit)
constexpr int kRtHashCols = 1024;    // distinct columns a block may have for the hashed fill
// shared memory of one build warp: the keys (or the hash table) and the column list
constexpr size_t kRtBuildSlice = (size_t)kRtMaxEnt * 8 + (size_t)kRtHashCols * 4;
constexpr int kRtBuildWarps = 4;
// staging of the gathered T_n rows (the kernel's STAGE parameter)
constexpr int kRtRegs = 0;     // registers, fragments exchanged by shuffles
constexpr int kRtCpAsync = 1;  // shared-memory ring filled by cp.async (16 bytes a lane)
constexpr int kRtTma = 2;      // shared-memory ring filled by TMA row gathers (tile::gather4)

__device__ __forceinline__ void cp_async_cg16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Four 128-byte rows y0..y3 of the [n][32] FP32 tensor of `map` into 512 bytes
// of shared memory (rows at dst + 128 i, 16-byte chunk c of the row at address
// bits 4..6 = c ^ (address bits 7..9): the 128-byte swizzle), completion counted
// on `bar` in bytes.
__device__ __forceinline__ void tma_gather4(void* dst, const CUtensorMap* map, int y0, int y1, int y2, int y3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(y0), "r"(y1), "r"(y2), "r"(y3), "r"(smem_u32(bar))
      : "memory");
}

// Arrival with the byte count of the copies to come, without release
// semantics: the producer publishes nothing of its own through the barrier
// (the copies' bytes are made visible by their completion), so the arrival
// need not wait for this lane's earlier memory operations (its matrix copies
// in flight).
__device__ __forceinline__ void mbar_expect_tx_relaxed(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.relaxed.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

struct RtArgs {
  CUtensorMap tmap;  // kRtTma: T_n as [n][32] FP32, boxes of one 128-byte row, 128-byte swizzle
  int64_t n;    // rows
  int64_t nrb;  // row blocks
  const unsigned char* __restrict__ data;  // k-steps in processing order
  const int64_t* __restrict__ wbeg;        // [grid * W + 1] first k-step of each warp
  const int64_t* __restrict__ kst;         // [blocks] k-steps of each block
  const float* __restrict__ tn;
  float* __restrict__ tp;
  const float* __restrict__ tprev;  // null: T_{n-1} is read from tp
  int first;
  float alpha;  // 0: the default (1 for the first step, else 2)
  double* __restrict__ partials;
  const double* __restrict__ prev_partials;
  double* __restrict__ prev_dots;
  int group;        // G: consecutive blocks per run
  int chunk;        // consecutive tiles per CTA between grid-wide jumps
  // kRtTma: row waits give up after spin_limit polls or two seconds and set *status
  uint64_t spin_limit;
  int* status;
  int never_wait;   // test hook: the warps first wait on a barrier nothing completes
};

}  // namespace

namespace {

// ---------------------------------------------------------------- the step kernels

// FP32 products from TF32 units: x = hi + lo with hi = x with its low 13
// mantissa bits cleared (a TF32 value) and lo = x - hi (exact); the tensor core
// reads the TF32 bits of each operand (the top 19) and ignores the rest, so lo
// enters truncated. The product is taken as lo*hi + hi*lo + hi*hi; the dropped
// lo*lo term and the truncation of lo leave a relative error below 2^-20. The
// hi*hi terms and the two cross terms go to separate FP32 accumulators (four
// independent MMA chains per k-step), summed at the block's end.
// The A operand of one k-step (chunk cg of the T_n rows of slots t and t + 4)
// split into TF32 high and low parts; shared by the n-tiles of a 16-row block.
struct RtA {
  uint32_t ah[8], al[8];
  __device__ __forceinline__ void split(const float4& fa, const float4& fb) {
    constexpr uint32_t m = 0xffffe000u;
    const float xs[8] = {fa.x, fa.y, fa.z, fa.w, fb.x, fb.y, fb.z, fb.w};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      ah[i] = __float_as_uint(xs[i]) & m;
      al[i] = __float_as_uint(xs[i] - __uint_as_float(ah[i]));
    }
  }
};

struct RtAcc {
  float h0[4], h1[4], l0[4], l1[4];  // m-tiles 0 (logical columns 0..15) and 1 (16..31)
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < 4; ++i) h0[i] = h1[i] = l0[i] = l1[i] = 0.f;
  }
  // A: the split rows; (vx, vy) = (V[g][t], V[g][t+4]) of this n-tile's rows
  __device__ __forceinline__ void mma(const RtA& A, float vx, float vy) {
    constexpr uint32_t m = 0xffffe000u;
    const uint32_t bh0 = __float_as_uint(vx) & m, bh1 = __float_as_uint(vy) & m;
    const uint32_t bl0 = __float_as_uint(vx - __uint_as_float(bh0));
    const uint32_t bl1 = __float_as_uint(vy - __uint_as_float(bh1));
    // logical columns g, g + 8 (m-tile 0) and g + 16, g + 24 (m-tile 1)
    mma_tf32(l0, A.al[0], A.al[1], A.al[4], A.al[5], bh0, bh1);
    mma_tf32(l1, A.al[2], A.al[3], A.al[6], A.al[7], bh0, bh1);
    mma_tf32(h0, A.ah[0], A.ah[1], A.ah[4], A.ah[5], bh0, bh1);
    mma_tf32(h1, A.ah[2], A.ah[3], A.ah[6], A.ah[7], bh0, bh1);
    mma_tf32(l0, A.ah[0], A.ah[1], A.ah[4], A.ah[5], bl0, bl1);
    mma_tf32(l1, A.ah[2], A.ah[3], A.ah[6], A.ah[7], bl0, bl1);
  }
  // fa, fb: chunk cg of the T_n rows of slots t and t + 4; v: (V[g][t], V[g][t+4])
  __device__ __forceinline__ void add(const float4& fa, const float4& fb, const float2& v) {
    RtA A;
    A.split(fa, fb);
    mma(A, v.x, v.y);
  }
  // rows 2t and 2t + 1 of the n-tile, memory columns 4 cg .. 4 cg + 3
  __device__ __forceinline__ void rows(float4& r0, float4& r1) const {
    r0 = make_float4(h0[0] + l0[0], h0[2] + l0[2], h1[0] + l1[0], h1[2] + l1[2]);
    r1 = make_float4(h0[1] + l0[1], h0[3] + l0[3], h1[1] + l1[1], h1[3] + l1[3]);
  }
};

__device__ __forceinline__ int2 ld_stream_i2(const void* p) {
  int2 r;
  asm volatile("ld.global.nc.L1::no_allocate.v2.s32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "l"(p));
  return r;
}
__device__ __forceinline__ float2 ld_stream_f2(const void* p) {
  float2 r;
  asm volatile("ld.global.nc.L1::no_allocate.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "l"(p));
  return r;
}

// One kernel, three ways of staging the gathered T_n rows:
//  - STAGE = kRtCpAsync: cp.async copies into a per-warp shared-memory ring (see
//    the file comment) D = XS - 1 k-steps ahead, the matrix data MS - 1 ahead;
//    both rings are powers of two and the main loop is unrolled over the matrix
//    ring, so every slot is a compile-time constant;
//  - STAGE = kRtTma: the same pipeline, but lane 0 fetches the 8 rows of a
//    k-step with two TMA row gathers (tile::gather4, 4 rows of 128 bytes each),
//    completion counted on the entry's mbarrier. Each gather lands on a 1 KB
//    boundary, where the 128-byte swizzle of the tensor map puts chunk c of row
//    r at c ^ r, the layout the cp.async form writes by hand, so the fragment
//    reads are the same. The gathers leave the load/store pipe out of the row
//    copies, but a warp's iteration then carries an mbarrier arrive, two tensor
//    copies and a wait (each a few hundred cycles of latency even when the data
//    is there), and 4-row gathers top out near 4.5 TB/s per GPU at 16 warps:
//    1.2 ms against 0.65 ms on a 2.4M-orbital flake. Kept as a tested option.
//    Waits are bounded: after spin_limit polls or two seconds the warp records
//    a timeout in *status, drains the gathers it issued and stops;
//  - STAGE = kRtRegs: no shared memory, so the whole L1 caches T_n rows. Lane (q, p)
//    loads 16-byte chunk p of the T_n rows of slots q and q + 4 (one 128-byte row
//    per quarter-warp, one L1 wavefront per slot) D k-steps ahead into registers,
//    and the A fragments are gathered from those registers with eight shuffles
//    per k-step (lane (g, t) takes chunk cg of slots t and t + 4 from lane
//    8t + cg). The matrix stream is read with loads that skip L1: the columns 2D
//    k-steps ahead (they address the row loads), the values D ahead.
// Either way the matrix stream is prefetched into L2 in bulk further ahead.
// Each warp walks its blocks in the build's processing order: runs of G
// consecutive blocks, run i in tile (bid + (i / chunk) grid) chunk + i % chunk;
// a block ends after its k-step count (kst), read one block ahead.
// The epilogue's reads of T_n and T_{n-1} rows: through the read-only path, or,
// in a launch that runs several steps (COH), from L2, since other CTAs of the
// launch wrote those rows after L1 may have cached older ones.
template <bool COH>
__device__ __forceinline__ float4 ld_rows_tn(const float* p) {
  if constexpr (COH) return __ldcg(reinterpret_cast<const float4*>(p));
  else return ldg4(p);
}
template <bool COH>
__device__ __forceinline__ float4 ld_rows_tprev(const float* p) {
  if constexpr (COH) return __ldcg(reinterpret_cast<const float4*>(p));
  else return ld_once4(p);
}

// CPX: a complex H~ on blocks of 8 rows, stored with the 16-row k-step layout
// (R = 16): n-tile 0 holds the real parts of the values, n-tile 1 the imaginary
// parts. A complex vector is a (re, im) column pair, so with X the gathered
// rows, the products P_re = X Re(V)^T and P_im = X Im(V)^T give
//   (H X)_re = P_re[re col] - P_im[im col],  (H X)_im = P_re[im col] + P_im[re col],
// combined in the lane's own four columns (two pairs) at the block's end.
template <int W, int D, int STAGE, int R, bool COH = false, bool CPX = false>
__device__ __forceinline__ void rt_body(const RtArgs& a, const int bid, const int nblk) {
  constexpr bool REGS = STAGE == kRtRegs;
  constexpr int NTI = R / kRtRows;       // n-tiles (8 rows each) of the k-step panel
  constexpr int RB = CPX ? kRtRows : R;  // rows of a block
  constexpr int NTR = RB / kRtRows;      // n-tiles of the block's rows
  static_assert(!CPX || R == 16, "complex blocks: 8 rows in the 16-row k-step layout");
  constexpr int KB = rt_step_bytes(R);   // bytes of one k-step
  static_assert((R == 8 || R == 16) && (R == 8 || STAGE == kRtCpAsync), "16-row blocks: cp.async form only");
  static_assert(!COH || STAGE == kRtCpAsync, "multi-step launches: the cp.async form (its gathers bypass L1)");
  constexpr int C = 32;
  constexpr int NT = W * 32;
  constexpr int XS = D + 1;      // shared ring of staged T_n rows (k-steps)
  constexpr int MS = 2 * XS;     // shared ring of matrix k-steps
  constexpr int DM = MS - 1 - D; // matrix lookahead beyond the rows'
  constexpr int kPf = REGS ? 48 : 32;  // matrix k-steps prefetched into L2 ahead
  constexpr int kDotFlush = 16;        // blocks summed in FP32 between FP64 flushes
  static_assert(REGS || ((XS & (XS - 1)) == 0 && DM >= D + 1), "power-of-two rings, matrix ahead of the rows");
  extern __shared__ __align__(1024) unsigned char rt_smem_raw[];
  // the 128-byte swizzle of TMA copies is a function of the address: ring
  // entries sit on 1 KB boundaries (the launch adds 1 KB of slack)
  unsigned char* rt_smem = rt_smem_raw + ((1024u - (smem_u32(rt_smem_raw) & 1023u)) & 1023u);
  if (a.prev_partials) reduce_prev<C, NT>(a.prev_partials, a.prev_dots, nblk, bid, nblk);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3, q = lane >> 3, p = lane & 7;
  const int cg = (g >> 1) | ((g & 1) << 2);  // the lane's chunk of 4 memory columns
  const int64_t n = a.n;
  const int first = a.first, group = a.group, chunk = a.chunk;
  const float alpha = a.alpha != 0.f ? a.alpha : (first ? 1.f : 2.f);
  const float* tprev = a.tprev ? a.tprev : a.tp;
  float* tp = a.tp;
  const float* tnc = a.tn + 4 * cg;
  const unsigned char* tnb = reinterpret_cast<const unsigned char*>(a.tn + 4 * p);  // + column * 128
  const int64_t* kst = a.kst;
  const int64_t k0 = a.wbeg[bid * W + warp];
  const int nk = (int)(a.wbeg[bid * W + warp + 1] - k0);
  const unsigned char* gdata = a.data + k0 * KB;

  // block walk, block-end countdown and epilogue operands
  // run i of the warp lies in tile (bid + (i / chunk) nblk) chunk + i % chunk;
  // the walk keeps that tile split as (tb, ic) for the run after the current
  // one, advanced without divisions
  int jb = 0;
  int64_t tb = (int64_t)bid * chunk;
  int ic = 0;
  auto run_row = [&]() -> int64_t { return ((tb + ic) * W + warp) * group * RB; };
  auto next_run = [&]() {
    if (++ic == chunk) {
      ic = 0;
      tb += (int64_t)nblk * chunk;
    }
  };
  int64_t rbase = run_row(), row0 = 0;  // first row of the current run
  next_run();
  int64_t nbase = run_row();  // first row of the next run
  int left = 0;                                       // k-steps of the current block still to run
  int next_left = nk > 0 ? (int)kst[rbase / RB] : 0;  // the next block's k-steps
  // T_n and T_{n-1} of the lane's rows 8 nt + 2t and 8 nt + 2t + 1 of the block
  float4 xn0[NTI], xn1[NTI], xp0[NTI], xp1[NTI];
#pragma unroll
  for (int nt = 0; nt < NTI; ++nt) xn0[nt] = xn1[nt] = xp0[nt] = xp1[nt] = make_float4(0.f, 0.f, 0.f, 0.f);
  // dots: FP32 over kDotFlush blocks, then FP64; lane (g, t) ends with column 4 cg + t
  double d0 = 0.0, d1 = 0.0;
  float e0[4], e1[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) e0[c] = e1[c] = 0.f;
  int since_flush = 0;
  auto flush = [&]() {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      e0[c] += __shfl_xor_sync(0xffffffffu, e0[c], 1);
      e1[c] += __shfl_xor_sync(0xffffffffu, e1[c], 1);
      e0[c] += __shfl_xor_sync(0xffffffffu, e0[c], 2);
      e1[c] += __shfl_xor_sync(0xffffffffu, e1[c], 2);
    }
    float v0 = e0[0], v1 = e1[0];
#pragma unroll
    for (int c = 1; c < 4; ++c)
      if (t == c) {
        v0 = e0[c];
        v1 = e1[c];
      }
    d0 += (double)v0;
    d1 += (double)v1;
#pragma unroll
    for (int c = 0; c < 4; ++c) e0[c] = e1[c] = 0.f;
  };
  auto begin_block = [&]() {
    row0 = rbase + (int64_t)jb * RB;
    left = next_left;
    // the k-steps of the block after this one (its run may start elsewhere)
    const int64_t nrow = jb + 1 < group ? row0 + RB : nbase;
    if (nrow / RB < a.nrb) next_left = (int)kst[nrow / RB];
#pragma unroll
    for (int nt = 0; nt < NTR; ++nt) {
      const int64_t r0 = row0 + 8 * nt + 2 * t;
      if (r0 < n) {
        xn0[nt] = ld_rows_tn<COH>(tnc + r0 * C);
        if (!first) xp0[nt] = ld_rows_tprev<COH>(tprev + r0 * C + 4 * cg);
      }
      if (r0 + 1 < n) {
        xn1[nt] = ld_rows_tn<COH>(tnc + (r0 + 1) * C);
        if (!first) xp1[nt] = ld_rows_tprev<COH>(tprev + (r0 + 1) * C + 4 * cg);
      }
    }
  };
  auto row_out = [&](int64_t r, const float4& h, const float4& xp, const float4& xn) {
    if (r >= n) return;
    const float4 y = first ? make_float4(alpha * h.x, alpha * h.y, alpha * h.z, alpha * h.w)
                           : make_float4(alpha * h.x - xp.x, alpha * h.y - xp.y, alpha * h.z - xp.z,
                                         alpha * h.w - xp.w);
    st_na4(tp + r * C + 4 * cg, y);
    e0[0] += xn.x * xn.x;
    e0[1] += xn.y * xn.y;
    e0[2] += xn.z * xn.z;
    e0[3] += xn.w * xn.w;
    e1[0] += y.x * xn.x;
    e1[1] += y.y * xn.y;
    e1[2] += y.z * xn.z;
    e1[3] += y.w * xn.w;
  };
  RtAcc acc[NTI];
#pragma unroll
  for (int nt = 0; nt < NTI; ++nt) acc[nt].zero();
  auto end_block = [&]() {
    if constexpr (CPX) {
      float4 a0, a1, b0, b1;  // real-part and imaginary-part products, rows 2t and 2t + 1
      acc[0].rows(a0, a1);
      acc[1].rows(b0, b1);
      acc[0].zero();
      acc[1].zero();
      // memory columns 4 cg .. 4 cg + 3 are the pairs (4 cg, 4 cg + 1), (4 cg + 2, 4 cg + 3)
      const float4 h0 = make_float4(a0.x - b0.y, a0.y + b0.x, a0.z - b0.w, a0.w + b0.z);
      const float4 h1 = make_float4(a1.x - b1.y, a1.y + b1.x, a1.z - b1.w, a1.w + b1.z);
      const int64_t r0 = row0 + 2 * t;
      row_out(r0, h0, xp0[0], xn0[0]);
      row_out(r0 + 1, h1, xp1[0], xn1[0]);
    } else {
#pragma unroll
      for (int nt = 0; nt < NTI; ++nt) {
        float4 h0, h1;
        acc[nt].rows(h0, h1);
        acc[nt].zero();
        const int64_t r0 = row0 + 8 * nt + 2 * t;
        row_out(r0, h0, xp0[nt], xn0[nt]);
        row_out(r0 + 1, h1, xp1[nt], xn1[nt]);
      }
    }
    if (++jb == group) {
      jb = 0;
      rbase = nbase;
      next_run();
      nbase = run_row();
    }
    if (++since_flush == kDotFlush) {
      since_flush = 0;
      flush();
    }
  };
  // the MMAs of one k-step, with the block walk around them
  auto consume = [&](const float4& fa, const float4& fb, const float2& v) {
    if (left == 0) begin_block();
    acc[0].add(fa, fb, v);
    if (--left == 0) end_block();
  };

  if constexpr (STAGE == kRtCpAsync) {
    constexpr int kWarpBytes = XS * 1024 + MS * KB;
    constexpr int kChunks = KB / 16;  // 16-byte chunks of a matrix k-step (18 or 34)
    static_assert(MS % 8 == 0, "L2 prefetch every 8 matrix k-steps at fixed slots of the unrolled loop");
    unsigned char* xr = rt_smem + (size_t)warp * kWarpBytes;
    unsigned char* mr = xr + XS * 1024;
    // Lane (g, t) copies, and later reads, chunk cg of the T_n rows of slots t
    // and t + 4 (16-byte chunk c of row s at c ^ s: no bank conflicts either
    // way, and a quarter of the warp covers each 128-byte row). A lane reads
    // only rows it copied itself, so its own cp.async wait orders them; the
    // matrix k-steps (copied in 16-byte chunks by all lanes, read by all) are
    // ordered by one __syncwarp per iteration.
    const int ro0 = t * 128 + 16 * (cg ^ t), ro1 = 512 + t * 128 + 16 * (cg ^ (t + 4));
    // iteration u (matrix slot sm = u mod MS): wait for the copies of iteration
    // u - D (the rows of k-step u, matrix k-step u + DM), copy matrix k-step
    // u + D + DM and the rows of k-step u + D, run k-step u's MMAs. The matrix
    // source of the iteration is mb + off (mb: k-step u's chunk of this lane).
    auto iter = [&](int u, int sm, const unsigned char* mb, int off, bool checks, bool pf) {
      cp_async_wait<D - 1>();
      __syncwarp();  // every lane's matrix copies have landed; k-step u - 1 is read
      const int vm = u + D + DM, vx = u + D;
      if (!checks || vm < nk) {
        unsigned char* md = mr + ((sm + MS - 1) & (MS - 1)) * KB + 16 * lane;
        const unsigned char* msrc = mb + (off + (D + DM) * KB);
        if (lane < kChunks) cp_async_cg16(md, msrc);
        if (kChunks > 32 && lane < kChunks - 32) cp_async_cg16(md + 512, msrc + 512);
      }
      if (pf && lane == 0 && vm + kPf < nk)
        prefetch_l2_bulk(gdata + (size_t)(vm + kPf) * KB, (uint32_t)min(8, nk - vm - kPf) * KB);
      if (!checks || (vx >= 0 && vx < nk)) {
        // the columns of k-step vx (slots t, t + 4) landed DM iterations ago
        const int2 cc = *reinterpret_cast<const int2*>(mr + ((sm + D) & (MS - 1)) * KB + 8 * t);
        unsigned char* dst = xr + ((sm + D) & (XS - 1)) * 1024;
        cp_async_cg16(dst + ro0, tnc + (uint64_t)(uint32_t)cc.x * C);
        cp_async_cg16(dst + ro1, tnc + (uint64_t)(uint32_t)cc.y * C);
      }
      cp_async_commit();
      if (checks && u < 0) return;
      const unsigned char* xs = xr + (sm & (XS - 1)) * 1024;
      const unsigned char* ms = mr + sm * KB;
      RtA A;
      A.split(*reinterpret_cast<const float4*>(xs + ro0), *reinterpret_cast<const float4*>(xs + ro1));
      if constexpr (NTI == 1) {
        const float2 v = *reinterpret_cast<const float2*>(ms + 32 + 8 * lane);
        acc[0].mma(A, v.x, v.y);
      } else {
        // (V[g][t], V[g][t+4]) of n-tile 0, then of n-tile 1
        const float4 v = *reinterpret_cast<const float4*>(ms + 32 + 16 * lane);
        acc[0].mma(A, v.x, v.y);
        acc[1].mma(A, v.z, v.w);
      }
      if (--left == 0) {
        end_block();
        if (u + 1 < nk) begin_block();
      }
    };
    if (nk > 0) begin_block();
    const unsigned char* mlan = gdata + 16 * lane;  // this lane's chunk of matrix k-step 0
    int u = -(D + DM);
    for (; u < 0; ++u) iter(u, u & (MS - 1), mlan, u * KB, true, (((u + D + DM) & 7) == 0));
    const int main_end = nk - (D + DM) > 0 ? ((nk - (D + DM)) & ~(MS - 1)) : 0;
    for (; u < main_end; u += MS) {
      const unsigned char* mb = mlan + (size_t)u * KB;
#pragma unroll
      for (int j = 0; j < MS; ++j) iter(u + j, j, mb, j * KB, false, ((j + D + DM) & 7) == 0);
    }
    for (; u < nk; ++u)
      iter(u, u & (MS - 1), mlan, u * KB, true, (((u + D + DM) & 7) == 0));
    cp_async_wait<0>();
  } else if constexpr (STAGE == kRtTma) {
    // Each warp owns XS entries of 2 KB (1 KB aligned): row entry e holds slots
    // 0..3 of its k-step at [0, 512) and slots 4..7 at [1024, 1536), each the
    // target of one gather on a 1 KB boundary, so the swizzle puts chunk c of
    // row r at c ^ r (r = 0..3); matrix slot m sits in the hole after a half,
    // at 2048 (m >> 1) + 512 + 1024 (m & 1). Then one mbarrier per row entry.
    unsigned char* xr = rt_smem + (size_t)warp * XS * 2048;
    unsigned char* mr = xr + 512;
    auto mslot = [&](int m) { return mr + (m >> 1) * 2048 + (m & 1) * 1024; };
    uint64_t* bars = reinterpret_cast<uint64_t*>(rt_smem + (size_t)W * XS * 2048) + warp * XS;
    if (lane == 0) {
#pragma unroll
      for (int i = 0; i < XS; ++i) mbar_init(&bars[i], 1);
      mbar_fence_init();
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncwarp();
    const bool mlane = lane < kRtStepBytes / 16;
    const unsigned char* msrc = gdata + 16 * lane;  // this lane's chunk of matrix k-step u + D + DM
    // reads of slot t and t + 4, chunk cg, in the swizzled entry
    const int ro0 = t * 128 + 16 * (cg ^ t), ro1 = 1024 + t * 128 + 16 * (cg ^ t);
    constexpr int kLogXS = XS == 4 ? 2 : XS == 8 ? 3 : XS == 2 ? 1 : 4;
    static_assert((1 << kLogXS) == XS, "row ring of 2, 4, 8 or 16 entries");
    bool gave_up = false;
    int stop = nk;  // first k-step not consumed
    if (a.never_wait && !bounded_wait(&bars[0], 0u, a.spin_limit)) {
      // test hook: nothing arrives on the entry, no copy was issued
      if (lane == 0) atomicExch(a.status, leo2d::kStatusTimeout);
      gave_up = true;
      stop = 0;
    }
    // iteration u (matrix slot sm = u mod MS): copy matrix k-step u + D + DM,
    // gather the rows of k-step u + D (their columns landed DM iterations ago),
    // wait for k-step u's rows, run its MMAs. Returns false after a timeout.
    auto iter = [&](int u, int sm, bool checks) -> bool {
      __syncwarp();  // every lane is done with the entries these copies overwrite
      const int vm = u + D + DM, vx = u + D;
      if (mlane && (!checks || vm < nk)) cp_async_cg16(mslot((sm + MS - 1) & (MS - 1)) + 16 * lane, msrc);
      msrc += kRtStepBytes;
      if (lane == 0) {
        if ((vm & 7) == 0 && vm + kPf < nk)
          prefetch_l2_bulk(gdata + (size_t)(vm + kPf) * kRtStepBytes, (uint32_t)min(8, nk - vm - kPf) * kRtStepBytes);
        if (!checks || (vx >= 0 && vx < nk)) {
          const int4* cp = reinterpret_cast<const int4*>(mslot((sm + D) & (MS - 1)));
          const int4 c0 = cp[0], c1 = cp[1];  // slots (0 4 1 5), (2 6 3 7)
          const int e = (sm + D) & (XS - 1);
          unsigned char* dst = xr + e * 2048;
          // no proxy fence here: the entry's last reads fed the warp's mma.sync of
          // the previous iteration, so they completed before this copy is issued
          // (a fence would also wait for this lane's matrix copies in flight)
          mbar_expect_tx_relaxed(&bars[e], 1024);
          tma_gather4(dst, &a.tmap, c0.x, c0.z, c1.x, c1.z, &bars[e]);
          tma_gather4(dst + 1024, &a.tmap, c0.y, c0.w, c1.y, c1.w, &bars[e]);
        }
      }
      cp_async_commit();
      cp_async_wait<D>();  // matrix k-step u + DM - 1 has landed (columns of the next gather, values of u)
      __syncwarp();
      if (checks && u < 0) return true;
      const int e = sm & (XS - 1);
      const bool ok = bounded_wait(&bars[e], (uint32_t)(u >> kLogXS) & 1u, a.spin_limit);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) atomicExch(a.status, leo2d::kStatusTimeout);
        stop = u;
        return false;
      }
      const unsigned char* xs = xr + e * 2048;
      consume(*reinterpret_cast<const float4*>(xs + ro0), *reinterpret_cast<const float4*>(xs + ro1),
              *reinterpret_cast<const float2*>(mslot(sm) + 32 + 8 * lane));
      return true;
    };
    int u = -(D + DM);
    if (!gave_up)
      for (; u < 0; ++u) iter(u, u & (MS - 1), true);
    const int main_end = nk - (D + DM) > 0 ? ((nk - (D + DM)) & ~(MS - 1)) : 0;
    for (; !gave_up && u < main_end; u += MS) {
#pragma unroll
      for (int j = 0; j < MS; ++j)
        if (!iter(u + j, j, false)) {
          gave_up = true;
          break;
        }
    }
    for (; !gave_up && u < nk; ++u)
      if (!iter(u, u & (MS - 1), true)) gave_up = true;
    cp_async_wait<0>();
    if (gave_up) {
      // gathers issued for k-steps stop .. stop + D may still land: wait for them
      // (bounded by time) before the shared memory is released
      if (lane == 0)
        for (int v = stop; v < min(stop + D + 1, nk); ++v)
          if (v >= 0 && !a.never_wait) bounded_wait(&bars[v & (XS - 1)], (uint32_t)(v >> kLogXS) & 1u, ~0ull);
      __syncwarp();
    }
  } else {
    const int src = 8 * t + cg;  // the lane holding chunk cg of slots t and t + 4
    // rings (slot j = k-step mod D): columns of k-steps u + D .. u + 2D - 1, rows
    // and values of k-steps u .. u + D - 1
    int2 cc[D];
#pragma unroll
    for (int j = 0; j < D; ++j) cc[j] = make_int2(0, 0);
    float4 xa[D], xb[D];
    float2 vv[D];
    auto load_cols = [&](int v) { return ld_stream_i2(gdata + (size_t)v * kRtStepBytes + 8 * q); };
    auto issue = [&](int j, int v) {  // k-step v (its columns in cc[j]) into slot j
      const int2 c = cc[j];
      xa[j] = ldg4(reinterpret_cast<const float*>(tnb + (uint64_t)(uint32_t)c.x * (C * 4)));
      xb[j] = ldg4(reinterpret_cast<const float*>(tnb + (uint64_t)(uint32_t)c.y * (C * 4)));
      vv[j] = ld_stream_f2(gdata + (size_t)v * kRtStepBytes + 32 + 8 * lane);
    };
    if (lane == 0 && kPf < nk)
      prefetch_l2_bulk(gdata + (size_t)kPf * kRtStepBytes, (uint32_t)min(8, nk - kPf) * kRtStepBytes);
#pragma unroll
    for (int j = 0; j < D; ++j)
      if (j < nk) cc[j] = load_cols(j);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      if (j < nk) {
        issue(j, j);
        if (j + D < nk) cc[j] = load_cols(j + D);
      }
    }
    for (int u0 = 0; u0 < nk; u0 += D) {
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const int u = u0 + j;
        if (u >= nk) break;  // warp-uniform
        float4 fa, fb;
        fa.x = __shfl_sync(0xffffffffu, xa[j].x, src);
        fa.y = __shfl_sync(0xffffffffu, xa[j].y, src);
        fa.z = __shfl_sync(0xffffffffu, xa[j].z, src);
        fa.w = __shfl_sync(0xffffffffu, xa[j].w, src);
        fb.x = __shfl_sync(0xffffffffu, xb[j].x, src);
        fb.y = __shfl_sync(0xffffffffu, xb[j].y, src);
        fb.z = __shfl_sync(0xffffffffu, xb[j].z, src);
        fb.w = __shfl_sync(0xffffffffu, xb[j].w, src);
        const float2 v = vv[j];
        // the slot is free: k-step u + D goes into it, and the columns of u + 2D
        if (u + D < nk) {
          issue(j, u + D);
          if (u + 2 * D < nk) cc[j] = load_cols(u + 2 * D);
        }
        if (lane == 0 && ((u + D) & 7) == 0 && u + D + kPf < nk)
          prefetch_l2_bulk(gdata + (size_t)(u + D + kPf) * kRtStepBytes,
                           (uint32_t)min(8, nk - (u + D + kPf)) * kRtStepBytes);
        consume(fa, fb, v);
      }
    }
  }
  flush();
  // warps add their columns in warp order (deterministic)
  __shared__ double bsum[2 * C];
  for (int i = threadIdx.x; i < 2 * C; i += NT) bsum[i] = 0.0;
  __syncthreads();
  const int col = 4 * cg + t;
  for (int w = 0; w < W; ++w) {
    if (warp == w) {
      bsum[2 * col] += d0;
      bsum[2 * col + 1] += d1;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < 2 * C; i += NT) a.partials[(size_t)bid * 2 * C + i] = bsum[i];
}

template <int W, int D, int STAGE, int R = kRtRows, bool CPX = false>
__global__ void __launch_bounds__(W * 32, 1) k_cheb_rt(const __grid_constant__ RtArgs a) {
  rt_body<W, D, STAGE, R, false, CPX>(a, (int)blockIdx.x, (int)gridDim.x);
}

// ---------------------------------------------------------------- batched flakes, one launch

// Every Chebyshev step of one pass over a batch of flakes in a single
// cooperative launch: the CTAs of flake f (block_first[f] .. block_first[f+1])
// run the 8-row step on its blocks, then meet at the flake's barrier (a counter
// in global memory) before the next step; flakes never wait on one another.
// Step k reads T_k from one buffer and writes T_{k+1} over T_{k-1} in the other;
// its prologue reduces step k-1's partials into dots[k-1], as the per-step
// launches do. The barrier: __syncthreads, a GPU-scope fence and an atomic
// arrival by thread 0, which then polls the counter with acquire loads. Polls
// give up after spin_limit rounds or two seconds: the CTA records a timeout,
// raises the abort flag (which every polling CTA also reads) and leaves; its
// copies were all waited for at the end of its step.
struct RtBatchParams {
  leo2d::RtBatchFlake f[leo2d::kRtBatchMax];
  int block_first[leo2d::kRtBatchMax + 1];
  int nflakes, steps;
  unsigned* bar;    // [nflakes] arrivals, zero at launch
  int* abort;       // non-zero: some CTA gave up
  int* status;
  uint64_t spin_limit;
  int never_arrive; // test hook: barrier targets one arrival more than the group makes
};
static_assert(sizeof(RtBatchParams) <= 32764, "batched 8-row parameters exceed the parameter space");

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ bool rt_group_barrier(const RtBatchParams& p, unsigned* bar, unsigned target) {
  __shared__ int go;
  __syncthreads();  // every thread of the CTA is done with the step
  if (threadIdx.x == 0) {
    __threadfence();  // the CTA's T_{k+1} rows and partials, at GPU scope
    atomicAdd(bar, 1u);
    int ok = 1;
    const uint64_t t0 = umma::now_ns();
    for (uint64_t k = 0;; ++k) {
      if (ld_acquire_u32(bar) >= target) break;
      if (*reinterpret_cast<volatile int*>(p.abort) != 0) {
        ok = 0;
        break;
      }
      if (k >= p.spin_limit || ((k & 255) == 255 && umma::now_ns() - t0 > 2000000000ull)) {
        atomicExch(p.status, leo2d::kStatusTimeout);
        atomicExch(p.abort, 1);
        ok = 0;
        break;
      }
    }
    __threadfence();
    go = ok;
  }
  __syncthreads();
  return go != 0;
}

template <int W, int D>
__global__ void __launch_bounds__(W * 32, 1) k_cheb_rt_batch(const __grid_constant__ RtBatchParams p) {
  int f = 0;
  while (f + 1 < p.nflakes && (int)blockIdx.x >= p.block_first[f + 1]) ++f;
  const int bid = (int)blockIdx.x - p.block_first[f], nblk = p.block_first[f + 1] - p.block_first[f];
  const leo2d::RtBatchFlake& F = p.f[f];
  constexpr int C = 32;
  for (int k = 0; k < p.steps; ++k) {
    RtArgs a{};
    a.n = F.n;
    a.nrb = F.nrb;
    a.data = F.data;
    a.wbeg = F.wbeg;
    a.kst = F.kst;
    a.tn = k % 2 == 0 ? F.x0 : F.x1;
    a.tp = k % 2 == 0 ? F.x1 : F.x0;
    a.tprev = nullptr;
    a.first = k == 0;
    a.alpha = 0.f;
    a.partials = F.partials[k % 2];
    a.prev_partials = k == 0 ? nullptr : F.partials[(k + 1) % 2];
    a.prev_dots = k == 0 ? nullptr : F.dots + (size_t)(k - 1) * 2 * C;
    a.group = F.group;
    a.chunk = F.chunk;
    a.spin_limit = p.spin_limit;
    a.status = p.status;
    rt_body<W, D, kRtCpAsync, kRtRows, true>(a, bid, nblk);
    const unsigned target = (unsigned)(k + 1) * (unsigned)nblk + (p.never_arrive ? 1u : 0u);
    if (!rt_group_barrier(p, p.bar + f, target)) break;
  }
}

// ---------------------------------------------------------------- format build

// One warp per block of R rows, at most kRtMaxEnt stored entries; the distinct
// columns are the slots. Pass 0 counts them in a hash set in the warp's slice of
// shared memory and writes the k-steps of each block; pass 1 sorts the keys
// (column << 16 | entry index) in that slice and writes the block's k-steps at
// kstart[b] (data zero-filled before): the
// columns in the interleaved order, the values in fragment order (lane 4g + t
// holds V[g][t], V[g][t+4] of each n-tile of 8 rows in turn), entries of one
// (row, column) summed in entry order.
template <int R, bool CPX = false>
__global__ void __launch_bounds__(kRtBuildWarps * 32)
    k_rt_build(int64_t n, int64_t nrb, const int64_t* __restrict__ prow, const int32_t* __restrict__ pcol,
               const float* __restrict__ pval, const float* __restrict__ pim, int pass, int64_t* __restrict__ kst,
               const int64_t* __restrict__ kstart, unsigned char* __restrict__ data, int* __restrict__ err,
               unsigned long long* __restrict__ ssum) {
  extern __shared__ __align__(16) unsigned char rt_build_smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(rt_build_smem + (size_t)w * kRtBuildSlice);
  uint32_t* list = reinterpret_cast<uint32_t*>(rt_build_smem + (size_t)w * kRtBuildSlice + (size_t)kRtMaxEnt * 8);
  const int64_t warps = (int64_t)gridDim.x * kRtBuildWarps;
  // rows of a block: R, or 8 for a complex H (its values and imaginary parts in
  // n-tiles 0 and 1 of the 16-row k-step layout)
  constexpr int RB = CPX ? 8 : R;
  for (int64_t b = (int64_t)blockIdx.x * kRtBuildWarps + w; b < nrb; b += warps) {
    const int64_t r0 = b * RB;
    const int rows = (int)min((int64_t)RB, n - r0);
    const int64_t mine = lane <= RB ? prow[r0 + min(lane, rows)] : 0;
    int64_t srp[RB + 1];
#pragma unroll
    for (int k = 0; k <= RB; ++k) srp[k] = __shfl_sync(0xffffffffu, mine, k);
    auto srp_at = [&](int k) {
      int64_t v = srp[0];
#pragma unroll
      for (int kk = 1; kk <= RB; ++kk)
        if (k == kk) v = srp[kk];
      return v;
    };
    // row of the block holding entry e (offsets from the block's first entry)
    auto row_of = [&](int e) {
      int r = 0;
#pragma unroll
      for (int k = 1; k < RB; ++k) r += (k < rows && srp[k] - srp[0] <= e) ? 1 : 0;
      return r;
    };
    const int64_t q0 = srp[0];
    const int E = (int)(srp_at(rows) - q0);
    if (E > kRtMaxEnt) {
      if (lane == 0) {
        atomicOr(err, 1);
        if (pass == 0) kst[b] = 1;
      }
      continue;
    }
    __syncwarp();  // the previous block's keys are read
    if (pass == 0) {
      // counting needs the distinct columns only: a hash set in the warp's slice
      // (2 kRtMaxEnt 32-bit slots, load <= 1/2), no sort (was half the build)
      uint32_t* set = reinterpret_cast<uint32_t*>(keys);
      constexpr int kSet = 2 * kRtMaxEnt;
      for (int i = lane; i < kSet; i += 32) set[i] = 0xFFFFFFFFu;
      __syncwarp();
      int fresh = 0;
      for (int i = lane; i < E; i += 32) {
        const uint32_t c = (uint32_t)pcol[q0 + i];
        uint32_t h = (c * 2654435761u) & (kSet - 1);
        for (int probe = 0; probe < kSet; ++probe) {  // bounded: the set never fills
          const uint32_t prev = atomicCAS(&set[h], 0xFFFFFFFFu, c);
          if (prev == 0xFFFFFFFFu) {
            ++fresh;
            break;
          }
          if (prev == c) break;
          h = (h + 1) & (kSet - 1);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) fresh += __shfl_xor_sync(0xffffffffu, fresh, o);
      if (lane == 0) {
        kst[b] = max(1, (fresh + 7) / 8);
        atomicAdd(ssum, (unsigned long long)fresh);
        atomicMax(err + 1, fresh);
      }
      continue;
    }
    unsigned char* base = data + (size_t)kstart[b] * rt_step_bytes(R);
    auto col_at = [&](int s) {  // column entry of slot s
      const int jj = s & 7;
      return reinterpret_cast<int32_t*>(base + (size_t)(s >> 3) * rt_step_bytes(R)) + (jj < 4 ? 2 * jj : 2 * (jj - 4) + 1);
    };
    auto val_at = [&](int s, int r) {  // value of (row r, slot s)
      const int jj = s & 7;
      float* vp = reinterpret_cast<float*>(base + (size_t)(s >> 3) * rt_step_bytes(R) + 32);
      return vp + (4 * (r & 7) + (jj & 3)) * (R / 4) + 2 * (r >> 3) + (jj >> 2);
    };
    const int KS = (int)kst[b];
    if (8 * KS <= kRtHashCols) {
      // Hashed fill: a table of (column << 32 | slot << 16 | row mask) words holds
      // the distinct columns; only they are sorted (about 124 of the ~540 entries
      // of an 8-row block), and each entry finds its slot in the table. A
      // (row, column) pair stored twice falls through to the sort below, which
      // sums the pair in entry order.
      constexpr int kSet = kRtMaxEnt;  // 64-bit words; load <= 1/2
      constexpr unsigned long long kEmpty = ~0ull;
      for (int i = lane; i < kSet; i += 32) keys[i] = kEmpty;
      __syncwarp();
      auto find = [&](uint32_t c) {  // the table slot holding column c (present)
        uint32_t h = (c * 2654435761u) & (kSet - 1);
        for (int probe = 0; probe < kSet && (uint32_t)(keys[h] >> 32) != c; ++probe) h = (h + 1) & (kSet - 1);
        return h;
      };
      bool dup = false;
      for (int i = lane; i < E; i += 32) {
        const uint32_t c = (uint32_t)pcol[q0 + i];
        const unsigned long long bit = 1ull << row_of(i);
        uint32_t h = (c * 2654435761u) & (kSet - 1);
        for (int probe = 0; probe < kSet; ++probe) {  // bounded: the table never fills
          unsigned long long cur = keys[h];
          if (cur == kEmpty) {
            cur = atomicCAS(&keys[h], kEmpty, ((unsigned long long)c << 32) | bit);
            if (cur == kEmpty) break;
          }
          if ((uint32_t)(cur >> 32) == c) {
            if (atomicOr(&keys[h], bit) & bit) dup = true;
            break;
          }
          h = (h + 1) & (kSet - 1);
        }
      }
      if (!__any_sync(0xffffffffu, dup)) {
        __syncwarp();
        // the distinct columns, compacted in table order, then sorted
        constexpr int kPer = kSet / 32;
        int cnt = 0;
        for (int j = 0; j < kPer; ++j) cnt += keys[lane * kPer + j] != kEmpty ? 1 : 0;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        const int K = __shfl_sync(0xffffffffu, incl, 31);
        int at = incl - cnt;
        for (int j = 0; j < kPer; ++j) {
          const unsigned long long v = keys[lane * kPer + j];
          if (v != kEmpty) list[at++] = (uint32_t)(v >> 32);
        }
        int P2 = 32;
        while (P2 < K) P2 <<= 1;
        for (int i = K + lane; i < P2; i += 32) list[i] = 0xFFFFFFFFu;
        __syncwarp();
        for (int k = 2; k <= P2; k <<= 1)
          for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P2; i += 32) {
              const int ixj = i ^ j;
              if (ixj > i) {
                const bool up = (i & k) == 0;
                const uint32_t x = list[i], y = list[ixj];
                if ((x > y) == up) {
                  list[i] = y;
                  list[ixj] = x;
                }
              }
            }
            __syncwarp();
          }
        // slot s = the rank of its column; the table learns it
        for (int s2 = lane; s2 < K; s2 += 32) {
          const uint32_t c = list[s2];
          *col_at(s2) = (int32_t)c;
          const uint32_t h = find(c);
          keys[h] |= (unsigned long long)s2 << 16;
        }
        const int32_t pad_col = K > 0 ? (int32_t)list[0] : 0;
        for (int s2 = K + lane; s2 < 8 * KS; s2 += 32) *col_at(s2) = pad_col;
        __syncwarp();
        for (int i = lane; i < E; i += 32) {
          const uint32_t c = (uint32_t)pcol[q0 + i];
          const int s2 = (int)((keys[find(c)] >> 16) & 0xFFFFu);
          const int r = row_of(i);
          *val_at(s2, r) = pval[q0 + i];
          if constexpr (CPX) *val_at(s2, r + 8) = pim[q0 + i];
        }
        continue;
      }
      __syncwarp();  // the table is read; the sort below reuses the slice
    }
    int P2 = 32;
    while (P2 < E) P2 <<= 1;
    for (int i = lane; i < P2; i += 32)
      keys[i] = i < E ? (((unsigned long long)(uint32_t)pcol[q0 + i] << 16) | (unsigned long long)i) : ~0ull;
    __syncwarp();
    for (int k = 2; k <= P2; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < P2; i += 32) {
          const int ixj = i ^ j;
          if (ixj > i) {
            const bool up = (i & k) == 0;
            const unsigned long long x = keys[i], y = keys[ixj];
            if ((x > y) == up) {
              keys[i] = y;
              keys[ixj] = x;
            }
          }
        }
        __syncwarp();
      }
    // slot of each sorted entry: distinct columns counted in order (each lane a
    // contiguous range of the sorted keys)
    const int per = P2 / 32;
    const int i0 = lane * per;
    int cnt = 0;
    for (int j = 0; j < per; ++j) {
      const int i = i0 + j;
      if (i < E && (i == 0 || (keys[i] >> 16) != (keys[i - 1] >> 16))) ++cnt;
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int K = __shfl_sync(0xffffffffu, incl, 31);
    const int32_t pad_col = K > 0 ? (int32_t)(keys[0] >> 16) : 0;
    for (int s = K + lane; s < 8 * KS; s += 32) *col_at(s) = pad_col;
    int s = incl - cnt - 1;
    for (int j = 0; j < per; ++j) {
      const int i = i0 + j;
      if (i >= E) break;
      const unsigned long long k = keys[i];
      const uint32_t c = (uint32_t)(k >> 16);
      const int e = (int)(k & 0xFFFFu);
      const bool new_col = i == 0 || (keys[i - 1] >> 16) != c;
      if (new_col) {
        ++s;
        *col_at(s) = (int32_t)c;
      }
      const int r = row_of(e);
      // the first entry of each (column, row) run sums the run in entry order
      const bool run_start = new_col || row_of((int)(keys[i - 1] & 0xFFFFu)) != r;
      if (run_start) {
        float v = pval[q0 + e], vi = CPX ? pim[q0 + e] : 0.f;
        for (int i2 = i + 1; i2 < E; ++i2) {
          const unsigned long long k2 = keys[i2];
          if ((uint32_t)(k2 >> 16) != c) break;
          const int e2 = (int)(k2 & 0xFFFFu);
          if (row_of(e2) != r) break;
          v += pval[q0 + e2];
          if constexpr (CPX) vi += pim[q0 + e2];
        }
        *val_at(s, r) = v;
        if constexpr (CPX) *val_at(s, r + 8) = vi;
      }
    }
  }
}

__global__ void k_rt_gather_i64(const int32_t* __restrict__ seq, const int64_t* __restrict__ src, int64_t count,
                                int64_t* __restrict__ dst) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x)
    dst[j] = src[seq[j]];
}

__global__ void k_rt_scatter_i64(const int32_t* __restrict__ seq, const int64_t* __restrict__ pos, int64_t count,
                                 int64_t* __restrict__ dst) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x)
    dst[seq[j]] = pos[j];
}

__global__ void k_rt_warp_begin(const int64_t* __restrict__ first_pos, const int64_t* __restrict__ pos, int count,
                                int64_t* __restrict__ wbeg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    wbeg[i] = pos[first_pos[i]];
}

}  // namespace

// ---------------------------------------------------------------- host side

namespace {

struct RtShape {
  int64_t nrb, nruns, ntiles;
  unsigned grid;
};

RtShape rt_shape(const leo2d_ctx* ctx, int64_t n, int warps, int group, int chunk, int rows, int max_grid = 0) {
  RtShape s;
  s.nrb = (n + rows - 1) / rows;
  s.nruns = (s.nrb + group - 1) / group;
  s.ntiles = (s.nruns + warps - 1) / warps;
  const int64_t chunks = (s.ntiles + chunk - 1) / chunk;
  const int64_t cap = max_grid > 0 ? max_grid : (int64_t)ctx->sm_count;
  s.grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cap, chunks));
  return s;
}

// Shared memory of one warp's rings for row lookahead D (rows: D + 1 k-steps,
// matrix: 2 (D + 1) k-steps of blocks of `rows` rows): packed for cp.async; for
// TMA gathers 2 KB per row entry (the matrix in its holes) and its mbarrier.
constexpr int rt_warp_bytes(int depth, int stage, int rows) {
  return stage == kRtTma ? (depth + 1) * (2048 + 8) : (depth + 1) * 1024 + 2 * (depth + 1) * rt_step_bytes(rows);
}

// TMA maps of the T_n buffers a thread launched the TMA form on (three
// buffers rotate through a recursion): encoded once per (device, base, rows).
struct RtMapEntry {
  int device;
  const float* base;
  int64_t rows;
  CUtensorMap map;
};
thread_local std::vector<RtMapEntry> g_rt_maps;

const CUtensorMap& rt_tmap(int device, const float* base, int64_t rows) {
  for (const auto& e : g_rt_maps)
    if (e.device == device && e.base == base && e.rows == rows) return e.map;
  if (g_rt_maps.size() >= 16) g_rt_maps.erase(g_rt_maps.begin());
  RtMapEntry e;
  e.device = device;
  e.base = base;
  e.rows = rows;
  make_tmap_f32(&e.map, base, rows, 32, 32, 1);
  g_rt_maps.push_back(e);
  return g_rt_maps.back().map;
}

}  // namespace

namespace leo2d {

int rt_group_of(const leo2d_ctx* ctx) { return ctx->rt_group > 0 ? ctx->rt_group : 2; }
int rt_chunk_of(const leo2d_ctx* ctx) { return ctx->rt_chunk > 0 ? ctx->rt_chunk : 2; }

size_t rt_smem_bytes(int warps, int depth, int stage, int rows) {
  // shared-memory forms: 1 KB of slack to align the rings
  return stage == kRtRegs ? 0 : (size_t)warps * rt_warp_bytes(depth, stage, rows) + 1024;
}

unsigned rt_grid(leo2d_ctx* ctx, const leo2d_csr* csr, int warps, int rows) {
  return rt_shape(ctx, csr->n, warps, rt_group_of(ctx), rt_chunk_of(ctx), rows).grid;
}

void csr_drop_rt(leo2d_csr* csr) {
  csr->rt_counted = false;
  csr->rt_built = false;
  csr->rt_kst.release();
  csr->rt_wbeg.release();
  csr->rt_data.release();
  csr->rt_blocks = csr->rt_ksteps = csr->rt_union = 0;
  csr->rt_max_slots = 0;
  csr->rt_warps = csr->rt_group = csr->rt_chunk = 0;
  csr->rt_grid = 0;
  csr->rt_rows = 0;
}

bool csr_build_rt(leo2d_ctx* ctx, leo2d_csr* csr, int warps, int group, int chunk, int rows, int max_grid) {
  LEO_REQUIRE(csr->reordered, "the tensor-core row-block step needs the locality-ordered copy");
  LEO_REQUIRE(rows == 8 || rows == 16, "tensor-core row blocks hold 8 or 16 rows");
  const bool cpx = csr->complex_h;
  LEO_REQUIRE(!cpx || (rows == 8 && csr->pval_im32.p), "a complex Hamiltonian takes 8-row blocks");
  const int64_t n = csr->n;
  const int KB = rt_step_bytes(cpx ? 16 : rows);  // complex: real and imaginary panels
  const RtShape sh = rt_shape(ctx, n, warps, group, chunk, rows, max_grid);
  if (csr->rt_built && csr->rt_rows == rows && csr->rt_patch == csr->reorder_patch &&
      csr->rt_curve == csr->reorder_curve && csr->rt_warps == warps && csr->rt_group == group &&
      csr->rt_chunk == chunk && csr->rt_grid == sh.grid)
    return true;
  const size_t smem = (size_t)kRtBuildWarps * kRtBuildSlice;
  auto build_kernel = cpx ? k_rt_build<16, true> : rows == 16 ? k_rt_build<16> : k_rt_build<8>;
  LEO_CUDA(cudaFuncSetAttribute(build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned bgrid = grid_for(sh.nrb * 32, kRtBuildWarps * 32, (int64_t)ctx->sm_count * 8);
  DevBuf<int> err(2);
  DevBuf<unsigned long long> ssum(1);
  LEO_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), ctx->stream));
  LEO_CUDA(cudaMemsetAsync(ssum.p, 0, sizeof(unsigned long long), ctx->stream));
  if (!(csr->rt_counted && csr->rt_rows == rows && csr->rt_patch == csr->reorder_patch &&
        csr->rt_curve == csr->reorder_curve)) {
    csr_drop_rt(csr);
    csr->rt_kst.alloc(std::max<int64_t>(sh.nrb, 1));
    launch(ctx, "rt_build", [&] {
      build_kernel<<<bgrid, kRtBuildWarps * 32, smem, ctx->stream>>>(n, sh.nrb, csr->prow.p, csr->pcol.p,
                                                                       csr->pval32.p, nullptr, 0, csr->rt_kst.p,
                                                                       nullptr, nullptr, err.p, ssum.p);
    });
    int h[2] = {0, 0};
    unsigned long long hs = 0;
    d2h(ctx, h, err.p, 2);
    d2h(ctx, &hs, ssum.p, 1);
    ctx_sync(ctx);
    if (h[0] != 0) {
      csr_drop_rt(csr);
      return false;
    }
    csr->rt_counted = true;
    csr->rt_rows = rows;
    csr->rt_patch = csr->reorder_patch;
    csr->rt_curve = csr->reorder_curve;
    csr->rt_union = (int64_t)hs;
    csr->rt_max_slots = h[1];
    LEO_CUDA(cudaMemsetAsync(err.p, 0, 2 * sizeof(int), ctx->stream));
  }
  csr->rt_built = false;
  // processing order: CTA c, warp w, its runs (tile by tile), the blocks of a run
  std::vector<int32_t> seq;
  seq.reserve((size_t)sh.nrb);
  std::vector<int64_t> first((size_t)sh.grid * warps + 1);
  for (unsigned c = 0; c < sh.grid; ++c)
    for (int w = 0; w < warps; ++w) {
      first[(size_t)c * warps + w] = (int64_t)seq.size();
      for (int64_t i = 0;; ++i) {
        const int64_t tile = ((int64_t)c + (i / chunk) * (int64_t)sh.grid) * chunk + i % chunk;
        if (tile >= sh.ntiles) break;
        const int64_t run = tile * warps + w;
        if (run >= sh.nruns) break;
        for (int j = 0; j < group; ++j) {
          const int64_t b = run * group + j;
          if (b >= sh.nrb) break;
          seq.push_back((int32_t)b);
        }
      }
    }
  first[(size_t)sh.grid * warps] = (int64_t)seq.size();
  LEO_REQUIRE((int64_t)seq.size() == sh.nrb, "row-block order does not cover the matrix");
  DevBuf<int32_t> dseq(std::max<int64_t>(sh.nrb, 1));
  DevBuf<int64_t> kseq(std::max<int64_t>(sh.nrb, 1)), pos(sh.nrb + 1), dfirst(first.size());
  h2d(ctx, dseq.p, seq.data(), seq.size());
  h2d(ctx, dfirst.p, first.data(), first.size());
  const unsigned g = grid_for(sh.nrb, 256, (int64_t)ctx->sm_count * 16);
  launch(ctx, "rt_order", [&] { k_rt_gather_i64<<<g, 256, 0, ctx->stream>>>(dseq.p, csr->rt_kst.p, sh.nrb, kseq.p); });
  exclusive_scan_i64(ctx, kseq.p, pos.p, sh.nrb);
  int64_t total = 0;
  d2h(ctx, &total, pos.p + sh.nrb, 1);
  ctx_sync(ctx);
  DevBuf<int64_t> kstart(std::max<int64_t>(sh.nrb, 1));
  launch(ctx, "rt_order", [&] { k_rt_scatter_i64<<<g, 256, 0, ctx->stream>>>(dseq.p, pos.p, sh.nrb, kstart.p); });
  csr->rt_wbeg.alloc(first.size());
  launch(ctx, "rt_order", [&] {
    k_rt_warp_begin<<<grid_for((int64_t)first.size(), 256), 256, 0, ctx->stream>>>(dfirst.p, pos.p, (int)first.size(),
                                                                                   csr->rt_wbeg.p);
  });
  csr->rt_data.release();
  csr->rt_data.alloc((size_t)std::max<int64_t>(total, 1) * KB);
  LEO_CUDA(cudaMemsetAsync(csr->rt_data.p, 0, (size_t)std::max<int64_t>(total, 1) * KB, ctx->stream));
  launch(ctx, "rt_build", [&] {
    // pass 1 reads each block's k-step count (kst) and writes nothing to it
    build_kernel<<<bgrid, kRtBuildWarps * 32, smem, ctx->stream>>>(n, sh.nrb, csr->prow.p, csr->pcol.p,
                                                                     csr->pval32.p, cpx ? csr->pval_im32.p : nullptr,
                                                                     1, csr->rt_kst.p, kstart.p, csr->rt_data.p,
                                                                     err.p, ssum.p);
  });
  int h0 = 0;
  d2h(ctx, &h0, err.p, 1);
  ctx_sync(ctx);
  LEO_REQUIRE(h0 == 0, "row-block build: a block exceeds the entry limit after counting");
  csr->rt_blocks = sh.nrb;
  csr->rt_ksteps = total;
  csr->rt_warps = warps;
  csr->rt_group = group;
  csr->rt_chunk = chunk;
  csr->rt_grid = sh.grid;
  csr->rt_built = true;
  return true;
}

unsigned rt_batch_cap(leo2d_ctx* ctx, const leo2d_csr* csr) {
  return rt_shape(ctx, csr->n, kRtBatchWarps, rt_group_of(ctx), rt_chunk_of(ctx), kRtRows).grid;
}

size_t rt_batch_smem() { return rt_smem_bytes(kRtBatchWarps, kRtBatchDepth, kRtCpAsync, kRtRows); }

void rt_batch_prepare(leo2d_ctx* ctx, unsigned grid) {
  auto kern = k_cheb_rt_batch<kRtBatchWarps, kRtBatchDepth>;
  const size_t smem = rt_batch_smem();
  LEO_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0, coop = 0;
  LEO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kRtBatchWarps * 32, smem));
  LEO_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
  LEO_REQUIRE(coop != 0, "batched 8-row step: the device has no cooperative launches");
  LEO_REQUIRE(occ >= 1 && grid <= (unsigned)(occ * ctx->sm_count),
              "batched 8-row step: the CTAs of one launch cannot all be resident");
}

void rt_batch_launch(leo2d_ctx* ctx, const RtBatchFlake* fl, const int* block_first, int nflakes, int steps,
                     unsigned* bar, int* abort, int never_arrive) {
  LEO_REQUIRE(nflakes >= 1 && nflakes <= kRtBatchMax, "a batched launch holds 1..64 matrices");
  RtBatchParams p{};
  for (int f = 0; f < nflakes; ++f) p.f[f] = fl[f];
  for (int f = 0; f <= nflakes; ++f) p.block_first[f] = block_first[f];
  p.nflakes = nflakes;
  p.steps = steps;
  p.bar = bar;
  p.abort = abort;
  p.status = ctx->status.p;
  p.spin_limit = ctx->spin_limit;
  p.never_arrive = never_arrive;
  const unsigned grid = (unsigned)block_first[nflakes];
  const size_t smem = rt_batch_smem();
  auto kern = k_cheb_rt_batch<kRtBatchWarps, kRtBatchDepth>;
  LEO_REQUIRE(grid <= (unsigned)ctx->sm_count, "batched 8-row step: more CTAs than SMs");
  LEO_CUDA(cudaMemsetAsync(bar, 0, sizeof(unsigned) * nflakes, ctx->stream));
  LEO_CUDA(cudaMemsetAsync(abort, 0, sizeof(int), ctx->stream));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kRtBatchWarps * 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // every CTA resident at once: the barriers need it
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  launch(ctx, "cheb_batch_step", [&] { LEO_CUDA(cudaLaunchKernelEx(&cfg, kern, p)); });
}

void rt_launch_step(leo2d_ctx* ctx, const leo2d_csr* csr, const StepShape& shape, unsigned grid, size_t smem,
                    const float* tn, float* tp, const float* tprev, int first, float alpha, double* partials,
                    const double* prev_partials, double* prev_dots) {
  LEO_REQUIRE(csr->rt_built && csr->rt_warps == shape.rt_warps && csr->rt_grid == grid &&
                  csr->rt_rows == shape.rt_rows,
              "tensor-core row blocks built for another launch shape");
  LEO_REQUIRE(smem >= rt_smem_bytes(shape.rt_warps, shape.rt_depth, shape.rt_stage,
                                    csr->complex_h ? 16 : shape.rt_rows),
              "tensor-core row-block step: shared memory changed since setup");
  RtArgs a{};
  if (shape.rt_stage == kRtTma) {
    LEO_REQUIRE(csr->n < (1ll << 31), "TMA row gathers take int32 row coordinates");
    a.tmap = rt_tmap(ctx->device, tn, csr->n);
  }
  a.spin_limit = ctx->spin_limit;
  a.status = ctx->status.p;
  a.never_wait = ctx->test_unsatisfied_wait;
  a.n = csr->n;
  a.nrb = csr->rt_blocks;
  a.data = csr->rt_data.p;
  a.wbeg = csr->rt_wbeg.p;
  a.kst = csr->rt_kst.p;
  a.tn = tn;
  a.tp = tp;
  a.tprev = tprev;
  a.first = first;
  a.alpha = alpha;
  a.partials = partials;
  a.prev_partials = prev_partials;
  a.prev_dots = prev_dots;
  a.group = csr->rt_group;
  a.chunk = csr->rt_chunk;
  auto go = [&](auto kern, int warps) {
    LEO_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // the register form keeps no dynamic shared memory: the carveout goes to L1
    if (smem == 0) LEO_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 0));
    launch(ctx, "cheb_step", [&] { kern<<<grid, warps * 32, smem, ctx->stream>>>(a); });
  };
  const int key = shape.rt_warps * 10 + shape.rt_depth;
  if (csr->complex_h) {
    if (shape.rt_stage == kRtCpAsync && shape.rt_rows == 8)
      switch (key) {
        case 123: return go(k_cheb_rt<12, 3, kRtCpAsync, 16, true>, 12);
        case 163: return go(k_cheb_rt<16, 3, kRtCpAsync, 16, true>, 16);
      }
    fail(LEO2D_ERR_BAD_ARG,
         "complex 8-row step: shared memory by cp.async (stage 1), warps 12 or 16, depth 3");
  }
  if (shape.rt_rows == 16) {
    if (shape.rt_stage == kRtCpAsync)
      switch (key) {
        case 123: return go(k_cheb_rt<12, 3, kRtCpAsync, 16>, 12);
        case 163: return go(k_cheb_rt<16, 3, kRtCpAsync, 16>, 16);
      }
    fail(LEO2D_ERR_BAD_ARG, "16-row blocks: shared memory by cp.async (stage 1), warps 12 or 16, depth 3");
  }
  if (shape.rt_stage == kRtRegs) {
    switch (key) {
      case 162: return go(k_cheb_rt<16, 2, kRtRegs>, 16);
      case 163: return go(k_cheb_rt<16, 3, kRtRegs>, 16);
      case 164: return go(k_cheb_rt<16, 4, kRtRegs>, 16);
      case 124: return go(k_cheb_rt<12, 4, kRtRegs>, 12);
      case 126: return go(k_cheb_rt<12, 6, kRtRegs>, 12);
      case 86: return go(k_cheb_rt<8, 6, kRtRegs>, 8);
    }
    fail(LEO2D_ERR_BAD_ARG, "8-row step in registers: warps 16 (depth 2, 3, 4), 12 (4, 6) or 8 (6)");
  }
  if (shape.rt_stage == kRtTma) {
    switch (key) {
      case 87: return go(k_cheb_rt<8, 7, kRtTma>, 8);
      case 127: return go(k_cheb_rt<12, 7, kRtTma>, 12);
      case 163: return go(k_cheb_rt<16, 3, kRtTma>, 16);
    }
    fail(LEO2D_ERR_BAD_ARG, "8-row step by TMA gathers: warps 8 or 12 (depth 7) or 16 (depth 3)");
  }
  switch (key) {
    case 83: return go(k_cheb_rt<8, 3, kRtCpAsync>, 8);
    case 87: return go(k_cheb_rt<8, 7, kRtCpAsync>, 8);
    case 123: return go(k_cheb_rt<12, 3, kRtCpAsync>, 12);
    case 127: return go(k_cheb_rt<12, 7, kRtCpAsync>, 12);
    case 163: return go(k_cheb_rt<16, 3, kRtCpAsync>, 16);
    case 203: return go(k_cheb_rt<20, 3, kRtCpAsync>, 20);
    case 243: return go(k_cheb_rt<24, 3, kRtCpAsync>, 24);
  }
  fail(LEO2D_ERR_BAD_ARG, "8-row step in shared memory: warps 8 or 12 (depth 3 or 7), 16, 20 or 24 (depth 3)");
}

}  // namespace leo2d

extern "C" leo2d_status leo2d_csr_rt_info(const leo2d_csr* csr, int64_t* row_blocks, int64_t* ksteps,
                                          int64_t* union_slots, int32_t* max_slots) {
  if (!csr) return LEO2D_ERR_BAD_ARG;
  const bool b = csr->rt_built;
  if (row_blocks) *row_blocks = b ? csr->rt_blocks : 0;
  if (ksteps) *ksteps = b ? csr->rt_ksteps : 0;
  if (union_slots) *union_slots = b ? csr->rt_union : 0;
  if (max_slots) *max_slots = b ? csr->rt_max_slots : 0;
  return LEO2D_OK;
}
