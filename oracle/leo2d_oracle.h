/*
 * leo2d_oracle.h - CPU restatement of LEO2D's KPM path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker, never the product: only the
 * tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * Every function follows the reference function cited beside it, in FP64 on
 * the host, with 64-bit sizes and heap storage (the reference keeps int32 nnz
 * and stack arrays, src/matrix/spmatrix.h:39-47, src/locality.cpp:5965).
 *
 * Parity of this restatement is pinned against fixtures generated from the
 * reference's own sources (oracle/Makefile.ref -> oracle/_ref/, fixtures in
 * tests/golden/, generator tests/golden/make_golden.py).
 */
#ifndef LEO2D_ORACLE_H
#define LEO2D_ORACLE_H

#include <stdint.h>

#include "../include/leo2d_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_h oracle_h;

/* Locality::setupSupercell type 1 and the material lattices (locality.cpp:130-293). */
int oracle_geom_prepare(leo2d_geom* g);

/* Geometry + pairs + CSR of one job with zero shifts (reference order, stored
 * zeros kept): Sheet::setIndex, Hstruct::getInterPairs/getIntraPairs,
 * setConfigPositions, generateRealH. Returns 0 on success. */
int oracle_build(const leo2d_geom* g, oracle_h** out);
void oracle_free(oracle_h* h);
void oracle_info(const oracle_h* h, int64_t* n, int64_t* nnz, int64_t* n_intra, int64_t* n_inter);
/* Any pointer may be NULL. Sizes: rowptr n+1, col/val/dx/dy nnz, grid 4n, pos 3n,
 * intra pairs 2*n_intra (+ t, sc 2*n_intra), inter pairs 2*n_inter (+ sc). */
void oracle_get(const oracle_h* h, int64_t* rowptr, int32_t* col, double* val, double* val_dx,
                double* val_dy, int32_t* index_to_grid, double* pos);
void oracle_get_pairs(const oracle_h* h, int32_t* intra_pairs, double* intra_t, int32_t* intra_sc,
                      int32_t* inter_pairs, int32_t* inter_sc);
/* Hstruct::getTargetList, solver type 1 (hstruct.cpp:1049-1079): center-cell orbitals. */
/* Hstruct::getShiftConfigs (hstruct.cpp:672-820): out[n][2]; returns 1 unless 2 sheets. */
int oracle_shift_configs(const oracle_h* h, double* out);
int64_t oracle_targets(const oracle_h* h, const int32_t* target_sheets, int32_t num_target_sheets,
                       int64_t* out, int64_t cap);

/* Locality::computeDosTraceKPM (locality.cpp:6138-6234), literal: vectors [R][n]. */
void oracle_kpm_trace(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val,
                      int32_t R, const double* vectors, int32_t P, double* mu_out);
/* Same recursion with every moment from the doubling identities
 * (mu_{2k} = 2<T_k|T_k> - mu_0, mu_{2k+1} = 2<T_{k+1}|T_k> - mu_1), the form the
 * GPU kernel evaluates. */
void oracle_kpm_trace_doubling(int64_t n, const int64_t* rowptr, const int32_t* col,
                               const double* val, int32_t R, const double* vectors, int32_t P,
                               double* mu_out);
/* Complex Hamiltonian of a flake in a perpendicular field B (tesla), as
 * Locality::generateCpxH builds it (locality.cpp:4485-5310) without SOC or
 * k-sampling: every entry of the real H~ becomes std::polar(t, phi) with the
 * Peierls phase phi = 3.14e-5 B (x_col - x_row) (y_row + y_col) / 2
 * (Locality::peierlsPhase, locality.cpp:7157-7161). pos [n][3]. */
void oracle_peierls(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val,
                    const double* pos, double B, double* re, double* im);
/* Complex H~ of a k-sampled job, as generateCpxH builds it with the job's k_vec
 * (locality.cpp:4517-4524, 4885-4941): every pair of the built job becomes
 * std::polar(t, k.(r_col - r_row)) with r_row shifted into the pair's image,
 * summed per entry in pair order; the energy shift goes to the home image's
 * diagonal only. re/im [nnz] in the CSR order of oracle_get. */
void oracle_bloch(const oracle_h* h, double kx, double ky, double* re, double* im);
/* computeDosTraceKPM's complex branch (locality.cpp:6240-6346), literal: real
 * start vectors [R][n]. */
void oracle_kpm_trace_cpx(int64_t n, const int64_t* rowptr, const int32_t* col, const double* re,
                          const double* im, int32_t R, const double* vectors, int32_t P, double* mu_out);
/* computeDosKPM's complex branch (locality.cpp:6043-6136): unit start vectors. */
void oracle_kpm_ldos_cpx(int64_t n, const int64_t* rowptr, const int32_t* col, const double* re,
                         const double* im, const int64_t* targets, int64_t T, int32_t P, double* mu_out);
/* Complex recursion from complex start vectors (vre + i vim, [R][n]) with every
 * moment from the doubling identities mu_{2k} = 2<T_k|T_k> - mu_0,
 * mu_{2k+1} = 2 Re<T_{k+1}|T_k> - mu_1: the form the GPU kernel evaluates. */
void oracle_kpm_trace_cpx_doubling(int64_t n, const int64_t* rowptr, const int32_t* col, const double* re,
                                   const double* im, int32_t R, const double* vre, const double* vim,
                                   int32_t P, double* mu_out);
/* Locality::computeDosKPM (locality.cpp:5945-6036): unit start vectors at targets. */
void oracle_kpm_ldos(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val,
                     const int64_t* targets, int64_t T, int32_t P, double* mu_out);
/* Locality::computeCondKPM (locality.cpp:6348-6720) with start_p1 = 0: out [T][P][P],
 * row n (alpha side), column m (beta side). beta_{P-1}, which the reference
 * never writes, is taken as 0 here. */
void oracle_kpm_cond(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val,
                     const double* val_dx, const int64_t* targets, int64_t T, int32_t P,
                     double* out);
/* Trace form of the same moments with random vectors r_v ([R][n], real):
 * out[a][b] += <T_a (dxH r)| dxH T_b r>, a,b < M (FP64). */
void oracle_kpm_cond_trace(int64_t n, const int64_t* rowptr, const int32_t* col,
                           const double* val, const double* val_dx, int32_t R,
                           const double* vectors, int32_t M, double* out);

/* Param_tools::densityTransform / densityTransformTrace (param_tools.cpp:661-768). */
void oracle_dos_transform(const double* mu, int32_t P, int32_t num_sets, double rescale,
                          double shift, double scale, double* dos_out, double* energies_out);
/* Jackson-damped DOS on an arbitrary grid (see leo2d_dos_reconstruct). */
void oracle_dos_reconstruct(const double* mu, int32_t P, const double* E, int64_t nE,
                            double rescale, double center, double scale, double* out);
/* Param_tools::matrixResponseTransform (param_tools.cpp:838-905), real case. */
void oracle_cond_transform(const double* M, int32_t P, double* out);
/* Diagonal of the Kubo-Greenwood form on an energy grid (see leo2d_cond_sigma). */
void oracle_cond_sigma(const double* mu, int32_t M, const double* E, int64_t nE, double rescale,
                       double center, double scale, double* out);

/* Vacancies, as workerChebSolve relabels orbitals (locality.cpp:2989-3016):
 * reduction[i] = number of listed orbitals below i (0-based; duplicates and
 * entries outside [0, n) count nothing), reduction[n] = total; returns the kept
 * count. */
int64_t oracle_vacancy_reduction(int64_t n, const int64_t* orbitals, int64_t count, int64_t* reduction);
/* generateRealH's vacancy skips (locality.cpp:3970-4010, 4215-4220, 4188,
 * 4305): rows of removed orbitals and entries in their columns are dropped, kept
 * columns become col - reduction[col]. Up to three value arrays (NULL skips one)
 * are carried. rp_out [kept + 1]; col/val outputs sized nnz. Returns the kept nnz. */
int64_t oracle_remove_orbitals(int64_t n, const int64_t* rowptr, const int32_t* col, const double* v0,
                               const double* v1, const double* v2, const int64_t* reduction,
                               int64_t* rp_out, int32_t* col_out, double* v0_out, double* v1_out,
                               double* v2_out);

/* Gershgorin bounds (FP64). */
void oracle_gershgorin(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val,
                       double* emin, double* emax);

/* Philox4x32-10 random-phase vectors, FP32-rounded, as the GPU generates them:
 * re/im [R][n]. */
void oracle_phase_vectors(uint64_t seed, uint64_t first_vector, int32_t R, int64_t n, double* re,
                          double* im);
/* The reference's trace vectors (locality.cpp:2274-2305): std::default_random_engine,
 * std::normal_distribution<double>(0,1), drawn vector by vector. */
void oracle_reference_gaussian(int32_t R, int64_t n, double* out);

#ifdef __cplusplus
}
#endif

#endif
