/*
 * cpu_baseline.cpp - the reference's CPU recursion, timed on host cores.
 *
 * TEST INFRASTRUCTURE ONLY (bench.py's cpu_baseline leg and its reference arm).
 * The work per Chebyshev step is what Locality::computeDosTraceKPM does per
 * vector (src/locality.cpp:6195-6234): one FP64 SpMV with the in-tree loop
 * (src/matrix/spmatrix.cpp:346-360), the three-term update and the two
 * doubling dot products. The reference runs one vector per MPI job and gets no
 * threads of its own (no OpenMP, MKL absent); here disjoint vector sets run on
 * `threads` host threads, standing in for one MPI worker per core.
 */
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <thread>
#include <vector>

extern "C" {

/* Runs `steps` Chebyshev steps on `nvec` real vectors of length n and returns
 * the wall time in seconds. Vectors are split across `threads` threads. The
 * checksum of the last moments is written to *checksum so the work cannot be
 * optimised away. */
double oracle_cpu_kpm_steps(int64_t n, const int64_t* rp, const int32_t* col, const double* val,
                            int32_t nvec, int32_t steps, int32_t threads, double* checksum) {
  if (threads < 1) threads = 1;
  std::vector<double> sums(nvec, 0.0);
  auto work = [&](int v0, int v1) {
    std::vector<double> Tp(n), Tj(n), Tn(n);
    for (int v = v0; v < v1; ++v) {
      for (int64_t i = 0; i < n; ++i) {
        Tj[i] = (double)((i * 2654435761u + v) % 1000) / 1000.0 - 0.5;
        Tp[i] = 0.0;
      }
      double acc = 0.0;
      for (int s = 0; s < steps; ++s) {
        for (int64_t r = 0; r < n; ++r) {
          double temp_sum = 0;
          for (int64_t i = rp[r]; i < rp[r + 1]; ++i) temp_sum += Tj[col[i]] * val[i];
          Tn[r] = 2 * temp_sum + 0 * Tn[r];
        }
        double an_an = 0, anp_an = 0;
        for (int64_t c = 0; c < n; ++c) {
          Tn[c] = Tn[c] - Tp[c];
          an_an += Tj[c] * Tj[c];
          anp_an += Tn[c] * Tj[c];
        }
        acc += an_an + anp_an;
        Tp.swap(Tj);
        Tj.swap(Tn);
      }
      sums[v] = acc;
    }
  };
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  const int nt = threads < nvec ? threads : nvec;
  for (int t = 0; t < nt; ++t) {
    int v0 = (int)((int64_t)nvec * t / nt), v1 = (int)((int64_t)nvec * (t + 1) / nt);
    th.emplace_back(work, v0, v1);
  }
  for (auto& x : th) x.join();
  auto t1 = std::chrono::steady_clock::now();
  double cs = 0;
  for (double s : sums) cs += s;
  if (checksum) *checksum = cs;
  return std::chrono::duration<double>(t1 - t0).count();
}

/* H~ = (H + shift I) / rescale in place (generateRealH's rescale,
 * src/locality.cpp:4166-4176): the diagonal entries get the shift. */
void oracle_rescale_csr(int64_t n, const int64_t* rp, const int32_t* col, double* val, double rescale,
                        double shift) {
  for (int64_t r = 0; r < n; ++r)
    for (int64_t i = rp[r]; i < rp[r + 1]; ++i) val[i] = ((col[i] == r ? shift : 0.0) + val[i]) / rescale;
}

/* The doubling recursion of the oracle (oracle_kpm_trace_doubling: T_{k+1} =
 * 2 H T_k - T_{k-1}, mu_{2k} = 2 <T_k|T_k> - mu_0, mu_{2k+1} = 2 <T_{k+1}|T_k> -
 * mu_1) with each SpMV split over `threads` row ranges. Every row is summed in
 * the same order as the serial loop and the dots are serial, so the moments
 * equal the serial oracle's bit for bit. */
void oracle_kpm_trace_doubling_threads(int64_t n, const int64_t* rp, const int32_t* col, const double* val,
                                       int32_t R, const double* vectors, int32_t P, int32_t threads,
                                       double* mu_out) {
  if (threads < 1) threads = 1;
  std::vector<double> Tp(n), Tj(n), Tn(n);
  auto spmv = [&](const double* in, double* out, double alpha) {
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
      th.emplace_back([&, t] {
        for (int64_t r = n * t / threads; r < n * (t + 1) / threads; ++r) {
          double temp_sum = 0;
          for (int64_t i = rp[r]; i < rp[r + 1]; ++i) temp_sum += in[col[i]] * val[i];
          out[r] = alpha * temp_sum + 0 * out[r];
        }
      });
    for (auto& x : th) x.join();
  };
  for (int t = 0; t < R; ++t) {
    const double* v = vectors + (size_t)t * n;
    double* mu = mu_out + (size_t)t * P;
    for (int64_t i = 0; i < n; ++i) Tj[i] = v[i];
    std::fill(Tp.begin(), Tp.end(), 0.0);
    std::fill(Tn.begin(), Tn.end(), 0.0);
    for (int k = 0; k < P / 2; ++k) {
      spmv(Tj.data(), Tn.data(), k == 0 ? 1.0 : 2.0);
      if (k > 0)
        for (int64_t c = 0; c < n; ++c) Tn[c] -= Tp[c];
      double d0 = 0, d1 = 0;
      for (int64_t c = 0; c < n; ++c) {
        d0 += Tj[c] * Tj[c];
        d1 += Tn[c] * Tj[c];
      }
      if (k == 0) {
        mu[0] = d0;
        mu[1] = d1;
      } else {
        mu[2 * k] = 2 * d0 - mu[0];
        mu[2 * k + 1] = 2 * d1 - mu[1];
      }
      Tp.swap(Tj);
      Tj.swap(Tn);
    }
  }
}

}  // extern "C"
