/*
 * Direct-summation REDFT01 (DCT-III) behind the fftw3.h stand-in.
 * TEST INFRASTRUCTURE ONLY. Sums run in long double; the result matches an
 * FFT-based DCT-III to rounding.
 */
#include "fftw3.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

struct leo2d_fftw_plan_s {
  int dims;  // 1, 2, or -1 for the unsupported r2c plan
  int n0, n1;
  double* in;
  double* out;
};

namespace {

// out_k = in_0 + 2 * sum_{j=1}^{n-1} in_j cos(pi j (k + 1/2) / n), stride s
void redft01(int n, const double* in, long double* out, int stride_in) {
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int k = 0; k < n; ++k) {
    long double acc = in[0];
    for (int j = 1; j < n; ++j)
      acc += 2.0L * in[(size_t)j * stride_in] *
             std::cos(pi * (long double)j * ((long double)k + 0.5L) / (long double)n);
    out[k] = acc;
  }
}

}  // namespace

fftw_plan fftw_plan_r2r_1d(int n, double* in, double* out, fftw_r2r_kind kind,
                           unsigned) {
  if (kind != FFTW_REDFT01) return nullptr;
  return new leo2d_fftw_plan_s{1, n, 1, in, out};
}

fftw_plan fftw_plan_r2r_2d(int n0, int n1, double* in, double* out,
                           fftw_r2r_kind k0, fftw_r2r_kind k1, unsigned) {
  if (k0 != FFTW_REDFT01 || k1 != FFTW_REDFT01) return nullptr;
  return new leo2d_fftw_plan_s{2, n0, n1, in, out};
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double*, fftw_complex*, unsigned) {
  return new leo2d_fftw_plan_s{-1, n0, n1, nullptr, nullptr};
}

void fftw_execute(const fftw_plan p) {
  if (!p || p->dims < 0) {
    std::fprintf(stderr, "fftw stub: plan kind not supported by the oracle\n");
    std::abort();
  }
  if (p->dims == 1) {
    std::vector<long double> o(p->n0);
    redft01(p->n0, p->in, o.data(), 1);
    for (int k = 0; k < p->n0; ++k) p->out[k] = (double)o[k];
    return;
  }
  // separable 2-D transform, row-major [n0][n1]: along dim 1 then dim 0
  const int n0 = p->n0, n1 = p->n1;
  std::vector<double> tmp((size_t)n0 * n1);
  std::vector<long double> o(n0 > n1 ? n0 : n1);
  for (int i = 0; i < n0; ++i) {
    redft01(n1, p->in + (size_t)i * n1, o.data(), 1);
    for (int k = 0; k < n1; ++k) tmp[(size_t)i * n1 + k] = (double)o[k];
  }
  for (int k1 = 0; k1 < n1; ++k1) {
    redft01(n0, tmp.data() + k1, o.data(), n1);
    for (int k0 = 0; k0 < n0; ++k0) p->out[(size_t)k0 * n1 + k1] = (double)o[k0];
  }
}

void fftw_destroy_plan(fftw_plan p) { delete p; }
void* fftw_malloc(size_t n) { return std::malloc(n); }
void fftw_free(void* p) { std::free(p); }
