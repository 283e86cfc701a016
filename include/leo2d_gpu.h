/*
 * leo2d_gpu.h - C ABI of the GB300 implementation of LEO2D's Chebyshev
 * kernel-polynomial-method (KPM) path.
 *
 * The reference (LEO2D) has no plugin interface for this path. Its worker runs,
 * per job, three C++ calls (src/locality.cpp:3041-3148):
 *   Locality::generateRealH      (src/locality.h:157, src/locality.cpp:3900)
 *   Locality::computeDosKPM / computeDosTraceKPM
 *                                (src/locality.h:173-176, src/locality.cpp:5945, 6138)
 *   Locality::computeCondKPM     (src/locality.h:179, src/locality.cpp:6348)
 * followed by Param_tools::densityTransform / densityTransformTrace /
 * conductivityTransform (src/params/param_tools.h:16-81). The entry points
 * below replace those calls one for one; each names the reference interface
 * it stands in for.
 *
 * Rules (all entry points):
 *  - Every function returns a leo2d_status; no C++ exception crosses the ABI.
 *    The text of the last failure is leo2d_last_error(ctx).
 *  - Host buffers are owned by the caller and are complete when the call
 *    returns (calls synchronise the context's stream before returning).
 *  - One context = one CUDA device + one stream. A context may be used by one
 *    host thread at a time; use one context per thread.
 *  - Sizes and indices that can exceed 2^31 are 64-bit.
 *  - There is no CPU fallback: without a usable CUDA device every compute call
 *    fails with LEO2D_ERR_CUDA.
 */
#ifndef LEO2D_GPU_H
#define LEO2D_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LEO2D_ABI_VERSION 2
#define LEO2D_MAX_SHEETS 8

typedef enum {
  LEO2D_OK = 0,
  LEO2D_ERR_BAD_ARG = 1,     /* invalid argument (null pointer, size, poly_order % 4 != 0, ...) */
  LEO2D_ERR_OOM = 2,         /* device or host allocation failed */
  LEO2D_ERR_CUDA = 3,        /* CUDA runtime error or no device */
  LEO2D_ERR_TIMEOUT = 4,     /* a bounded device-side wait ran out */
  LEO2D_ERR_NONFINITE = 5,   /* NaN or Inf met in an input or a result */
  LEO2D_ERR_UNSUPPORTED = 6, /* a reference option this build does not implement */
  LEO2D_ERR_IO = 7           /* file could not be read or written */
} leo2d_status;

/* Tight-binding models. LEO2D_MODEL_REF is the reference's graphene
 * (src/materials/graphene.h:77-95, graphene.cpp:13-222). LEO2D_MODEL_SIMPLE is
 * nearest-neighbour graphene, a = 2.46 A, t = -2.7 eV, with interlayer
 * t(r) = 0.33 exp(-(r - 3.35)/0.45) eV for 3-D distance r < 8 A. */
typedef enum { LEO2D_MODEL_REF = 0, LEO2D_MODEL_SIMPLE = 1 } leo2d_model;

/* Geometry of one job: what main.cpp:75-911 collects into Sdata/Job_params and
 * Locality::setupSupercell (src/locality.cpp:130-293) completes. Fields marked
 * "derived" are filled by leo2d_geom_prepare(). */
typedef struct {
  int32_t num_sheets;          /* NUM_SHEETS, 1..LEO2D_MAX_SHEETS */
  int32_t model;               /* leo2d_model (MATERIAL = Graphene -> REF) */
  int32_t boundary_condition;  /* BOUNDARY_CONDITION: 0 = disk flake, 1 = periodic supercell */
  int32_t sc_search_size;      /* supercell images searched, default 1 (job_params.cpp:57) */
  int32_t supercell_m;         /* SUPERCELL_M_N (periodic only) */
  int32_t supercell_n;
  int32_t min_shape[LEO2D_MAX_SHEETS][2]; /* MINSIZE per sheet (grid cells) */
  int32_t max_shape[LEO2D_MAX_SHEETS][2]; /* MAXSIZE per sheet */
  double max_R[LEO2D_MAX_SHEETS];         /* disk radius, A (MAXSIZE or MAX_R) */
  double heights[LEO2D_MAX_SHEETS];       /* HEIGHT, A */
  double angles[LEO2D_MAX_SHEETS];        /* ANGLE in radians (derived for periodic) */
  double energy_rescale;                  /* H~ = (H + shift*I) / rescale, as generateRealH */
  double energy_shift;
  /* derived */
  double lattice[LEO2D_MAX_SHEETS][2][2];       /* unrotated lattice vectors a1, a2 */
  double sheet_supercell[LEO2D_MAX_SHEETS][2][2];
  int32_t sheet_sc_stride[LEO2D_MAX_SHEETS][2][2];
  double supercell[2][2];                       /* sheet 0's supercell (Job_params "supercell") */
  int32_t prepared;
  /* B_FIELD with USE_B_FIELD = 1 (tesla, perpendicular): when non-zero the
   * Hamiltonian is complex, each entry t e^{i phi} with the Peierls phase
   * phi = 3.14e-5 B (x_col - x_row)(y_row + y_col)/2 of Locality::peierlsPhase
   * (src/locality.cpp:7157-7161), as generateCpxH builds it
   * (src/locality.cpp:4485-5310). On a periodic supercell every image takes the
   * phase with the row's orbital shifted into that image, as generateCpxH does
   * (src/locality.cpp:4718-4738); that H~ is not Hermitian in this gauge. */
  double b_field;
  /* Bloch vector (1/A) of a k-sampled job (K_SAMPLING = 1, Job_params "k_vec",
   * locality.cpp:1615-1650): when non-zero the Hamiltonian is complex, each
   * periodic image's hopping t e^{i k.(r_col - r_row)} with r_row shifted into
   * that image, summed per entry, as generateCpxH does (locality.cpp:4896-4941).
   * The energy shift then goes to the home image's diagonal only. */
  double k_vec[2];
  /* The job's sheet shifts (Job_params "shifts", recursiveShiftCalc,
   * locality.cpp:1222-1269): sheet s moves by shifts[s][0] a1 + shifts[s][1] a2
   * of its rotated lattice (setConfigPositions, locality.cpp:3618-3642). As in
   * the reference, the pairs come from the unshifted geometry and the values,
   * dxH and the positions the matrix keeps from the shifted one. |shift| <= 1. */
  double shifts[LEO2D_MAX_SHEETS][2];
  /* E_FIELD with USE_E_FIELD = 1: every diagonal entry becomes
   * (H_ii + energy_shift + z_i E) / energy_rescale, the on-site term of
   * Locality::onSiteE (src/locality.cpp:7163-7166, 4166-4172). 0 = off. */
  double e_field;
  /* TRILAYER_SUPERCELL = 1 (Job_params "supercell_type" 3, three sheets): the
   * (M, N) cell of a helical trilayer, Locality::setupSupercell's type 3
   * (src/locality.cpp:401-532). Sheets 0, 1, 2 at -theta, 0, theta with
   * strides (N^2 - M^2, M^2 + 2MN; -(M^2 + 2MN), N^2 + 2MN),
   * (0, M^2 + MN + N^2; -(M^2 + MN + N^2), M^2 + MN + N^2) and
   * (M^2 - N^2, N^2 + 2MN; -(N^2 + 2MN), M^2 + 2MN); the job's cell is sheet
   * 0's. 0 = the bilayer rule of SUPERCELL_M_N (type 1). */
  int32_t trilayer_supercell;
} leo2d_geom;

typedef struct leo2d_ctx leo2d_ctx;
typedef struct leo2d_csr leo2d_csr;

/* ---------------------------------------------------------------- context */

/* Creates a context on CUDA device `device` with its own stream. */
leo2d_status leo2d_ctx_create(leo2d_ctx** out, int device);
leo2d_status leo2d_ctx_destroy(leo2d_ctx* ctx);
/* Message of the last failure on this context ("" if none). */
const char* leo2d_last_error(const leo2d_ctx* ctx);
const char* leo2d_status_string(leo2d_status s);
int leo2d_abi_version(void);
/* The context's cudaStream_t, for callers that enqueue their own work. */
void* leo2d_ctx_stream(leo2d_ctx* ctx);
/* Iteration limit of every device-side spin wait (0 = library default).
 * A wait that runs out makes the call return LEO2D_ERR_TIMEOUT. */
leo2d_status leo2d_ctx_set_spin_limit(leo2d_ctx* ctx, uint64_t iterations);
/* When enabled, kernels are bracketed by CUDA events on the context stream and
 * per-kernel launch counts and device times are kept. */
leo2d_status leo2d_ctx_set_profiling(leo2d_ctx* ctx, int enable);
leo2d_status leo2d_ctx_kernel_stats(leo2d_ctx* ctx, const char* kernel,
                                    int64_t* launches, double* total_ms);
leo2d_status leo2d_ctx_reset_stats(leo2d_ctx* ctx);
/* Total kernel launches made through this context since creation. */
int64_t leo2d_ctx_launch_count(const leo2d_ctx* ctx);
/* Tuning switches of a context. Keys: "step_kernel" (-1 = autotuned or the
 * default for the matrix; 0 = shared-memory tiles filled by bulk copies;
 * 1 = register streaming of the matrix; 2 = tensor-core tiles; 3 = row blocks of
 * 4 rows; 5 = row blocks of 8 or 16 rows on the tensor cores),
 * "tile_stages" (2..4 shared-memory stages of the tiled kernel, default 2),
 * "tile_chunk" (1..65536 consecutive row tiles per block between grid-wide
 * jumps, default 4), "rt_warps" / "rt_depth" / "rt_group" / "rt_chunk" (the
 * tensor-core row-block step: warps per CTA 8, 12, 16, 20 or 24; k-steps of T_n
 * rows in flight per warp 2, 3, 4, 6 with the rows in registers or 3, 7 in
 * shared memory; blocks per warp run 1..16, default 2; tiles per CTA between
 * grid-wide jumps 1..64, default 2; 0 = autotuned or default), "rt_stage"
 * (-1 = autotuned, 0 = the T_n rows staged in registers, 1 = in shared memory
 * by cp.async, 2 = in shared memory by TMA row gathers), "rt_rows" (rows per
 * block: 0 = autotuned, 8, or 16 with rt_stage 1, warps 12 or 16, depth 3),
 * "alloc_cap_mb" (the largest single device allocation a call on this context
 * may make, in MiB; a larger one fails with LEO2D_ERR_OOM and a message naming
 * its size; 0 = no limit, the default),
 * "reorder_curve" (1 = inside each patch of the locality ordering, orbitals go
 * by sheet and along a Hilbert curve of 1/32-patch cells, the default; 0 = by
 * the reference index), "tile_warps" (8 or 24 warps per block of the tiled
 * kernel; 0 = chosen per block width, the default), "reorder" (locality ordering of the streamed matrix:
 * -1 = automatic for >= 1e5 orbitals with positions, 0 = off, 1 = on),
 * "reorder_patch_dA" (patch edge of that ordering in tenths of A, default 160),
 * "kubo_velocity" (trace Kubo moments: -1 = dxH built inside the row-block
 * step from the flake's positions, the default where it applies; 0 = the
 * stored dxH), "kubo_chunk" (trace Kubo moments: T_m vectors held at once,
 * a multiple of 4; 0 = as many as device memory allows), "mlp_fused" (the
 * control variate's network over many sites: 1 = one persistent launch with
 * every activation on chip, the default; 0 = one GEMM per layer). */
leo2d_status leo2d_ctx_set_option(leo2d_ctx* ctx, const char* key, int64_t value);

/* ---------------------------------------------------------------- geometry */

/* Fills the derived fields of `g`: lattices, and for periodic jobs the
 * supercell vectors, strides and sheet angles of Locality::setupSupercell
 * type 1 (src/locality.cpp:153-293). Host-only. */
leo2d_status leo2d_geom_prepare(leo2d_geom* g);

/* ---------------------------------------------------------------- (a) assembly */

#define LEO2D_CSR_KEEP_ZEROS 0x1u /* keep every stored entry of generateRealH (bit-exact layout) */
#define LEO2D_CSR_WITH_DX 0x2u    /* also build dxH = (x_i - x_j) H_ij and dyH (locality.cpp:4182-4183) */

/* Builds H~ on the device from the geometry: site enumeration
 * (Sheet::setIndex, src/geom/sheet.cpp:217), intra- and interlayer pair
 * search (Sheet::getIntraPairs sheet.cpp:624, Hstruct::getInterPairs
 * src/geom/hstruct.cpp:298) and CSR assembly (Locality::generateRealH,
 * src/locality.cpp:3900-4321). With LEO2D_CSR_KEEP_ZEROS the row pointers and
 * column indices equal the reference's; without it entries whose value is
 * exactly 0 are dropped (the layout the KPM kernels stream). */
leo2d_status leo2d_build_csr(leo2d_ctx* ctx, const leo2d_geom* g, uint32_t flags,
                             leo2d_csr** out);
leo2d_status leo2d_csr_destroy(leo2d_csr* csr);
/* n = orbitals, nnz = stored entries, pair counts as the reference's
 * max_intra_pairs / max_inter_pairs (src/locality.cpp:946-947). */
leo2d_status leo2d_csr_info(const leo2d_csr* csr, int64_t* n, int64_t* nnz,
                            int64_t* n_intra_pairs, int64_t* n_inter_pairs);
/* Copies the CSR to host arrays (any pointer may be NULL to skip it). */
leo2d_status leo2d_csr_download(leo2d_ctx* ctx, const leo2d_csr* csr, int64_t* rowptr,
                                int32_t* col, double* val, double* val_dx, double* val_dy);
/* Imaginary parts of the stored entries (complex H: leo2d_geom.b_field != 0),
 * in the order of leo2d_csr_download's values; val is the real part there.
 * generateCpxH keeps std::complex<double> val_c (src/locality.cpp:4928-4941). */
leo2d_status leo2d_csr_download_imag(leo2d_ctx* ctx, const leo2d_csr* csr, double* val_im);
/* index_to_grid [n][4] = (i, j, orbital, sheet) as Hstruct::getIndexArray
 * (hstruct.cpp:69-110); pos [n][3] = i2pos of setConfigPositions
 * (locality.cpp:3618-3642, zero shifts). Either pointer may be NULL. */
leo2d_status leo2d_csr_geometry(leo2d_ctx* ctx, const leo2d_csr* csr, int32_t* index_to_grid,
                                double* pos);
/* Uploads a host CSR (e.g. one generateRealH built) for the KPM calls. val_dx and
 * pos may be NULL. Replaces SpMatrix::setup (src/matrix/spmatrix.cpp:154-175). */
leo2d_status leo2d_csr_upload(leo2d_ctx* ctx, int64_t n, int64_t nnz, const int64_t* rowptr,
                              const int32_t* col, const double* val, const double* val_dx,
                              const double* pos, leo2d_csr** out);
/* The matrix of a job with vacancies: the listed orbitals (0-based, `count`
 * entries; duplicates and indices outside [0, n) remove nothing) are removed with
 * their rows and columns, and the kept orbitals keep their order, renumbered:
 * orbital i becomes i - (removed orbitals below i). Values (real and imaginary),
 * dxH/dyH, positions and grid indices follow. The reference builds this matrix
 * directly for its vacancy solvers (SOLVER_TYPE = MLMC_VAC / VD_FILE):
 * workerChebSolve's relabelling (src/locality.cpp:2989-3016) and the skips of
 * generateRealH / generateCpxH (locality.cpp:3970-4010, 4215-4220, 4188, 4305).
 * A target t of the reference's numbering is row t - (removed orbitals below t)
 * (computeDosKPM, locality.cpp:5963). *out is a new matrix; src is unchanged. */
leo2d_status leo2d_csr_remove_orbitals(leo2d_ctx* ctx, const leo2d_csr* src, const int64_t* orbitals,
                                       int64_t count, leo2d_csr** out);
/* Gershgorin bounds of the stored matrix, FP64: emin = min_i (H_ii - sum_{j!=i}|H_ij|),
 * emax = max_i (H_ii + sum_{j!=i}|H_ij|). */
leo2d_status leo2d_csr_bounds(leo2d_ctx* ctx, const leo2d_csr* csr, double* emin, double* emax);
/* In place: H <- (H + shift*I) / rescale (FP64, as a product with the FP64
 * reciprocal of rescale, within an ulp of the quotient; then the FP32 copy is
 * refreshed). */
leo2d_status leo2d_csr_rescale(leo2d_ctx* ctx, leo2d_csr* csr, double rescale, double shift);

/* Per-orbital local stacking disregistry of a bilayer, out[n][2] in [0,1)^2:
 * Hstruct::getShiftConfigs (src/geom/hstruct.cpp:672-820), bit-exact. The
 * learned control variate's site feature. Needs a matrix built by
 * leo2d_build_csr with two sheets. */
leo2d_status leo2d_csr_shift_configs(leo2d_ctx* ctx, const leo2d_csr* csr, double* out);

/* ---------------------------------------------------------------- (b) KPM DOS */

typedef enum {
  LEO2D_VEC_PHASE = 0,    /* complex random-phase vectors e^{i phi}, phi ~ U[0,2pi) from Philox4x32-10 */
  LEO2D_VEC_HOST = 1,     /* real vectors supplied by the caller ([num_vectors][n], FP64) */
  LEO2D_VEC_GAUSSIAN = 2  /* real N(0,1) vectors, Box-Muller on Philox4x32-10 */
} leo2d_vec_kind;

typedef enum { LEO2D_FP32 = 0, LEO2D_FP64 = 1 } leo2d_precision;

typedef struct {
  int32_t poly_order;    /* P (POLY_ORDER); a multiple of 4 (main.cpp:914-917) */
  int32_t num_vectors;   /* R random vectors (KPM_TRACE_SAMPS) */
  int32_t vector_kind;   /* leo2d_vec_kind */
  int32_t precision;     /* leo2d_precision of the recursion; moments always sum in FP64 */
  int32_t block;         /* vector-block width in columns per SpMM pass; 0 = autotuned */
  int32_t rows_per_warp; /* 0 = autotuned */
  uint64_t seed;         /* Philox key; vector v uses counter (v, row) */
  uint64_t first_vector; /* index of the first vector (lets callers extend a run) */
} leo2d_kpm_cfg;

/* Stochastic-trace moments: mu_out[v][n] = <r_v| T_n(H~) |r_v> for v < R, n < P.
 * Same recursion and moment doubling as Locality::computeDosTraceKPM
 * (src/locality.cpp:6138-6346): T_{n+1} = 2 H~ T_n - T_{n-1},
 * mu_{2n} = 2<T_n|T_n> - mu_0, mu_{2n+1} = 2<T_{n+1}|T_n> - mu_1.
 * For LEO2D_VEC_HOST, host_vectors is [R][n] (the reference's kpm_trace_vectors). */
leo2d_status leo2d_kpm_dos(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                           const double* host_vectors, double* mu_out);
/* Site-resolved moments mu_out[t][n] = <e_t| T_n(H~) |e_t>, as
 * Locality::computeDosKPM (src/locality.cpp:5945-6136). */
leo2d_status leo2d_kpm_ldos(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                            const int64_t* targets, int64_t num_targets, double* mu_out);
/* Times the step kernel on this matrix for every vector-block width (8..128
 * columns), rows per warp slot and warps per block, and keeps the fastest
 * choice per width and the width that minimises the time of a run of
 * cfg->num_vectors vectors; later calls with block = 0 / rows_per_warp = 0 use
 * them. No counterpart in the reference (its SpMV has no tunable shape). */
leo2d_status leo2d_kpm_autotune(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                                int32_t* block_out, int32_t* rows_out);
/* The step kernel a leo2d_kpm_dos call with this cfg would run on this matrix:
 * *kernel = 0 tiled CSR gathers, 1 register-streaming gathers, 2 tensor cores,
 * 3 row blocks, 4 row blocks over shared-memory windows, 5 row blocks of 8 rows
 * on the tensor cores; *block = the
 * vector-block width in columns. Builds nothing and
 * launches nothing. No counterpart in the reference. */
leo2d_status leo2d_kpm_step_kernel(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                                   int32_t* kernel, int32_t* block);

/* Param_tools::densityTransform (param_tools.cpp:661-705) for one moment set, or
 * densityTransformTrace (707-768) when num_sets > 1 (mean over sets first):
 * Jackson kernel, DCT-III, division by pi*sqrt(a^2 - (E_k - b)^2) at the P
 * Chebyshev nodes E_k = shift + rescale*cos((k+1/2)pi/P), times `scale`.
 * energies_out (may be NULL) receives E_k. FP64, on the device. */
leo2d_status leo2d_dos_transform(leo2d_ctx* ctx, const double* mu, int32_t poly_order,
                                 int32_t num_sets, double rescale, double shift, double scale,
                                 double* dos_out, double* energies_out);
/* Jackson-damped DOS on an arbitrary energy grid (FP64):
 * dos(E) = scale * [g_0 mu_0 + 2 sum_n g_n mu_n T_n(x)] / (pi rescale sqrt(1-x^2)),
 * x = (E - center) / rescale; zero outside |x| < 1. mu is the mean moment set. */
leo2d_status leo2d_dos_reconstruct(leo2d_ctx* ctx, const double* mu, int32_t poly_order,
                                   const double* energies, int64_t num_energies, double rescale,
                                   double center, double scale, double* dos_out);

/* ---------------------------------------------------------------- batched flakes */

/* Many matrices (flakes or twist angles of uneven size) run together, the whole
 * run captured once in a CUDA graph. Stands in for the reference's farm of
 * independent jobs, each running Locality::computeDosTraceKPM on its own rank
 * (src/locality.cpp:2295-2309, 6138-6346). With 32-column passes over matrices
 * with positions (block 0 or 32, the locality ordering on), every step of a
 * pass runs in one cooperative launch of the 8-row tensor-core step, each
 * matrix on its own group of CTAs (step_kernel = 3: one launch per step of the
 * 4-row step); otherwise one launch per step over all matrices. Each matrix
 * must already be rescaled (leo2d_csr_rescale) and must outlive the batch.
 * cfg: random-phase vectors, FP32 recursion (FP64 moments); block /
 * rows_per_warp 0 = autotuned over the batch (block width, warps, rows per slot
 * timed on real batched steps). 1..64 matrices. */
typedef struct leo2d_batch leo2d_batch;
leo2d_status leo2d_batch_create(leo2d_ctx* ctx, const leo2d_csr* const* csrs, int32_t num,
                                const leo2d_kpm_cfg* cfg, leo2d_batch** out);
/* One replay: mu_out[f][v][n], f < num, v < cfg->num_vectors, n < poly_order, for
 * Philox vectors first_vector + v under key seed (the vectors leo2d_kpm_dos draws). */
leo2d_status leo2d_batch_run(leo2d_batch* b, uint64_t seed, uint64_t first_vector, double* mu_out);
/* The chosen shape (warps 16: the one-launch form), the grid of each launch and
 * the kernel launches in one replay. */
leo2d_status leo2d_batch_info(const leo2d_batch* b, int32_t* block_cols, int32_t* warps,
                              int32_t* rows_per_item, int32_t* grid, int64_t* launches_per_run);
leo2d_status leo2d_batch_destroy(leo2d_batch* b);

/* ---------------------------------------------------------------- tensor cores */

/* D[M][N] = A[M][K] * B[N][K]^T with BF16 inputs (raw bits, row-major, K
 * contiguous) and FP32 accumulation, on the tcgen05 tensor cores (TMA-staged
 * operands, TMEM accumulator). The learned control variate's forward and
 * backward passes run on this kernel with fused epilogues; this entry point
 * exposes the plain product (host buffers) so it can be checked on its own.
 * K must be a multiple of 8. No counterpart in the reference. */
leo2d_status leo2d_tc_gemm(leo2d_ctx* ctx, const uint16_t* a, const uint16_t* b, int64_t M, int64_t N,
                           int64_t K, float* d);
/* D[128][N] = A[128][K] * B[N][K]^T in FP32 (host buffers) from three TF32
 * tensor-core products per K step (hi*hi + hi*lo + lo*hi, about 22 significant
 * bits), A held in tensor memory and B written into shared memory by the
 * threads: the arithmetic of the tensor-core Chebyshev step, exposed on its own
 * so it can be checked. K in {32, 64, 96, 128}, N a multiple of 8 up to 256,
 * N*K <= 24576. No counterpart in the reference. */
/* Tensor-core tiles of a matrix (built on first use of the tensor-core step):
 * tile count (0 if not built), mean and largest window (distinct columns of a
 * 128-row tile) and most entries in one tile. */
leo2d_status leo2d_csr_tc_info(const leo2d_csr* csr, int64_t* tiles, double* mean_window, int32_t* max_window,
                               int32_t* max_tile_entries);
/* Row blocks of the locality-ordered copy (built by the first recursion that
 * runs the row-block step, step_kernel = 3 or autotuned): blocks of 4 rows
 * stored as the sorted union of their rows' columns with a dense 4 x slots
 * panel of FP32 values, so that one gathered T_n row serves 4 rows. Reports the
 * row-block count, slots stored (padded to multiples of 4 per block), distinct
 * slots before padding, the most slots of one block and the largest tile of 16
 * blocks in bytes; zeros when not built. Replaces, for the recursion only, the
 * CSR stream of SpMatrix::vectorMultiply (src/matrix/spmatrix.cpp:346-360). */
leo2d_status leo2d_csr_rb_info(const leo2d_csr* csr, int64_t* row_blocks, int64_t* slots, int64_t* union_slots,
                               int32_t* max_slots, int64_t* max_tile_bytes);
/* Blocks of 8 rows of the tensor-core step (built by the first recursion that
 * runs it, step_kernel = 5 or autotuned): each block's slots are the sorted
 * union of its rows' columns in k-steps of 8 (288 bytes: 8 columns and the
 * 8 x 8 FP32 value panel in MMA fragment order), stored in the order one launch
 * shape processes them. Reports the block count, k-steps stored, distinct slots
 * before padding and the most slots of one block; zeros when not built.
 * Replaces, for the recursion only, the CSR stream of SpMatrix::vectorMultiply
 * (src/matrix/spmatrix.cpp:346-360). */
leo2d_status leo2d_csr_rt_info(const leo2d_csr* csr, int64_t* row_blocks, int64_t* ksteps, int64_t* union_slots,
                               int32_t* max_slots);
leo2d_status leo2d_tc_gemm_tf32x3(leo2d_ctx* ctx, const float* a, const float* b, int64_t N, int64_t K, float* d);

/* ---------------------------------------------------------------- learned control variate */

/* A small MLP on the tensor cores: per-site features (disregistry, twist,
 * layer, sublattice: 16 columns, FP32) -> 3 x 256 GELU -> the site's first 256
 * Chebyshev moments. BF16 weights and activations, FP32 accumulation, FP32
 * master weights with Adam. Trained on site-resolved moments from
 * leo2d_kpm_ldos and used only as a control variate for the stochastic
 * trace. No counterpart in the reference. Feature rows passed in are [n][F]
 * FP32 with F <= 64 (zero padded to 64). */
typedef struct leo2d_mlp leo2d_mlp;
int64_t leo2d_mlp_param_count(void);
/* Parameters are one FP32 vector: W0 [256][64], b0 [256], W1 [256][256], b1,
 * W2, b2, W3, b3 (W_l row-major [out][in]). Initialised from `seed`. */
leo2d_status leo2d_mlp_create(leo2d_ctx* ctx, uint64_t seed, leo2d_mlp** out);
leo2d_status leo2d_mlp_destroy(leo2d_mlp* mlp);
leo2d_status leo2d_mlp_get_params(leo2d_mlp* mlp, float* out);
leo2d_status leo2d_mlp_set_params(leo2d_mlp* mlp, const float* in);
/* Per-moment weights w[256] of the squared-error loss (default 1). */
leo2d_status leo2d_mlp_set_loss_weights(leo2d_mlp* mlp, const float* w);
/* Loss (1/n) sum_r sum_j w_j (y_rj - t_rj)^2 and its gradient with respect to
 * every parameter (layout as the parameter vector) for one batch of n rows,
 * n a multiple of 64 up to 65536. Does not update the parameters. */
leo2d_status leo2d_mlp_grad(leo2d_mlp* mlp, const float* x, int32_t F, const float* t, int64_t n,
                            double* loss, float* grad);
/* `steps` Adam steps (lr, beta 0.9/0.999) on minibatches of `batch` rows
 * (multiple of 64) sampled with replacement from the n training rows; one
 * step is a CUDA graph replay. loss_hist (may be NULL) gets each step's loss. */
leo2d_status leo2d_mlp_train(leo2d_mlp* mlp, const float* x, int32_t F, const float* t, int64_t n,
                             int32_t steps, int32_t batch, float lr, uint64_t seed, double* loss_hist);
/* Predicted moments y[n][256]. */
leo2d_status leo2d_mlp_predict(leo2d_mlp* mlp, const float* x, int32_t F, int64_t n, float* y);
/* The 16 feature columns of every orbital of a bilayer matrix: x_out[n][16]. */
leo2d_status leo2d_mlp_site_features(leo2d_ctx* ctx, const leo2d_csr* csr, double twist_deg, float* x_out);
/* sum over all orbitals of the predicted moments, FP64 sum_out[256] (features
 * built on the device; no per-site output). */
leo2d_status leo2d_mlp_site_sum(leo2d_mlp* mlp, const leo2d_csr* csr, double twist_deg, double* sum_out);

/* Trace moments with the network as a control variate: mu_out[n] estimates
 * Tr T_n(H~) (the scale of leo2d_kpm_dos's per-vector moments) for n < P.
 * For n < 256 it is  w_n * CV_n + (1 - w_n) * PH_n  and for n >= 256 PH_n, where
 *   PH_n = mean over cfg->num_vectors random vectors of <r|T_n|r> (leo2d_kpm_dos;
 *          0 vectors gives PH = 0),
 *   CV_n = sum_i f_n(i) over every orbital (network) + N * mean over num_sites
 *          orbitals s drawn uniformly (splitmix64 stream of site_seed) of
 *          (<s|T_n|s> - f_n(s)) (exact unit-vector moments, leo2d_kpm_ldos).
 * Both parts are unbiased, so the combination is for any fixed weights w
 * (NULL: w = 1). parts_out (optional) = [3][256]: sum_i f, the site
 * correction, PH. Locality::computeDosTraceKPM (src/locality.cpp:6138-6346)
 * is the plain estimator this extends; the reference has no control variate. */
leo2d_status leo2d_kpm_dos_cv(leo2d_ctx* ctx, const leo2d_csr* csr, leo2d_mlp* mlp, const leo2d_kpm_cfg* cfg,
                              double twist_deg, int64_t num_sites, uint64_t site_seed, const double* weights,
                              double* mu_out, double* parts_out);

/* ---------------------------------------------------------------- (c) Kubo conductivity */

/* Two-index Chebyshev moments of the current-current correlation.
 * With targets (num_targets >= 1): Locality::computeCondKPM
 * (src/locality.cpp:6348-6727) for each target t, mu_out[t][n][m] =
 * < dxH T_n(H~) a_0 , T_m(H~) e_t >, a_0 = -dxH e_t (start_p1 = 0,
 * cond_poly_par = 0); column m = P-1, which the reference never writes, is 0.
 * Without targets (NULL): the stochastic trace mu_out[n][m] =
 * (1/R) sum_r Re <T_n J r | J T_m r> = Tr[J T_n J T_m] estimate, J = i dxH, over
 * cfg->num_vectors random-phase or Gaussian vectors. The recursion runs in
 * FP32; the moment GEMM accumulates in FP64 across K chunks. The per-target
 * form needs a matrix built with LEO2D_CSR_WITH_DX. The trace form on a
 * flake with its geometry builds dxH inside the row-block step,
 * (dxH)_ij = (x_i - x_j) H~_ij, and needs no stored dxH; elsewhere it needs
 * LEO2D_CSR_WITH_DX too. */
leo2d_status leo2d_kpm_cond(leo2d_ctx* ctx, const leo2d_csr* csr, const leo2d_kpm_cfg* cfg,
                            const int64_t* targets, int64_t num_targets, double* mu_out);
/* Param_tools::matrixResponseTransform (param_tools.cpp:838-905), real case:
 * 2-D DCT-III of 2 g_i g_j M_ij with Jackson g_i / sqrt(2); P x P in and out. */
leo2d_status leo2d_cond_transform(leo2d_ctx* ctx, const double* M, int32_t poly_order, double* out);
/* sigma_xx(E) on an energy grid from trace moments (Kubo-Greenwood, Jackson
 * kernel): scale * sum_nm h_n h_m g_n g_m mu_nm T_n(x) T_m(x) / (pi^2 (1-x^2)),
 * x = (E - center)/rescale, h_0 = 1, h_n = 2. No counterpart in the reference,
 * which stops at the transformed matrix. */
leo2d_status leo2d_cond_sigma(leo2d_ctx* ctx, const double* mu, int32_t poly_order,
                              const double* energies, int64_t num_energies, double rescale,
                              double center, double scale, double* sigma_out);

/* ---------------------------------------------------------------- driver */

/* `LEO2D file.in` for the KPM path (app/src/main.cpp:23): parses the input with
 * main.cpp's keyword rules, builds and solves the SQ job on `device` and writes
 * <JOB_NAME>.cheb (Param_tools::save, param_tools.cpp:19-316) and, when asked,
 * <JOB_NAME>_matrix.dat / _pos.dat (locality.cpp:4366-4448) into out_dir.
 * Options of other reference paths make it return LEO2D_ERR_UNSUPPORTED; the
 * reason is copied into msg. */
leo2d_status leo2d_run_input(const char* in_path, const char* out_dir, int device, char* msg,
                             size_t msg_len);
/* Host only: the geometry and job switches leo2d_run_input reads from a .in
 * file (main.cpp:75-911 rules). ints_out (may be NULL) receives 10 values:
 * solver_type, observable_type, poly_order, kpm_trace, kpm_trace_samps,
 * verbose_save, matrix_save, number of unsupported options, first target sheet
 * (0-based), NSHIFTS. Unsupported options are listed in msg. */
leo2d_status leo2d_parse_input(const char* in_path, leo2d_geom* geom_out, int32_t* ints_out, char* msg,
                               size_t msg_len);

/* ---------------------------------------------------------------- no device allocation */

/* Allocation-free variant of leo2d_kpm_dos (random-phase vectors, FP32
 * recursion). No counterpart in the reference: it exists for callers that may
 * not allocate device memory - code that runs while a stream is being captured
 * into a CUDA graph, or a host application whose device memory is entirely
 * owned by its own allocator and budget - so it calls no cudaMalloc, cudaFree
 * or allocating library routine and needs no context.
 * Inputs and output are device pointers owned by the caller: the H~ CSR
 * (rowptr[n+1], col[nnz], FP32 val[nnz]) and mu_out[num_vectors][poly_order]
 * (FP64), written as leo2d_kpm_dos writes its host buffer. Work is enqueued on
 * `stream` (a cudaStream_t, NULL for the legacy stream) and the call returns
 * without waiting; synchronise the stream before reading mu_out.
 * Scratch: one file-scope 32 MiB device array (held by every device that loads
 * the library until the process exits). The two vector blocks, block partials
 * and moment dots must fit in it: n * 64 bytes plus a few hundred KB, i.e. up to
 * about 5e5 orbitals. Larger problems return LEO2D_ERR_BAD_ARG.
 * The first call on a device looks up the array's device address with that
 * device current (set-up, once per device); make that first call before any
 * stream capture. All calls share the array: calls that overlap on the GPU
 * (other streams, other host threads) race and corrupt each other's results.
 * Status codes: LEO2D_ERR_BAD_ARG (null pointer, size, poly_order % 4 != 0,
 * problem too large), LEO2D_ERR_CUDA (no device, failed launch). */
leo2d_status leo2d_kpm_dos_noalloc(const int64_t* rowptr, const int32_t* col, const float* val,
                                   int64_t n, int32_t poly_order, int32_t num_vectors,
                                   uint64_t seed, uint64_t first_vector, double* mu_out,
                                   void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LEO2D_GPU_H */
