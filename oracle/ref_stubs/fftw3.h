/*
 * Minimal stand-in for the FFTW3 API calls made by LEO2D.
 *
 * TEST INFRASTRUCTURE ONLY. FFTW is not installed in this container, so the
 * reference's own src/params/param_tools.cpp is compiled against this header.
 * fftw_direct.cpp evaluates the real-to-real REDFT01 kind (DCT-III, as FFTW's
 * documentation defines it: out_k = in_0 + 2 sum_{j>=1} in_j cos(pi j (k+1/2)/n))
 * by direct summation, in 1-D and separably in 2-D. Planning never touches the
 * arrays (FFTW_MEASURE in the real library may overwrite them; see the oracle's
 * notes on param_tools.cpp:692).
 * The complex-to-real 2-D plan used by the momentum-space solver is declared
 * but aborts when executed: that path is not part of the KPM oracle.
 */
#ifndef LEO2D_ORACLE_FFTW3_STUB_H
#define LEO2D_ORACLE_FFTW3_STUB_H

#include <cstddef>

typedef double fftw_complex[2];
typedef struct leo2d_fftw_plan_s* fftw_plan;
typedef int fftw_r2r_kind;

#define FFTW_REDFT01 1
#define FFTW_MEASURE 0u
#define FFTW_ESTIMATE (1u << 6)

fftw_plan fftw_plan_r2r_1d(int n, double* in, double* out, fftw_r2r_kind kind,
                           unsigned flags);
fftw_plan fftw_plan_r2r_2d(int n0, int n1, double* in, double* out,
                           fftw_r2r_kind kind0, fftw_r2r_kind kind1,
                           unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out,
                               unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void* fftw_malloc(size_t n);
void fftw_free(void* p);

#endif
