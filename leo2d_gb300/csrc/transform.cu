// transform.cu - FP64 reconstruction of the DOS from Chebyshev moments.
//
// leo2d_dos_transform replaces Param_tools::densityTransform and
// densityTransformTrace (src/params/param_tools.cpp:661-768): Jackson kernel
// g_i = ((P-i) cos(pi i/P) + sin(pi i/P) cot(pi/P)) / P, then FFTW's REDFT01
// (DCT-III, out_k = in_0 + 2 sum_{j>=1} in_j cos(pi j (k+1/2)/P)) evaluated as a
// direct sum, one thread per output node, cos(pi * j(2k+1)/(2P)) taken with
// cospi on the exactly reduced rational argument.
// leo2d_dos_reconstruct evaluates the same damped series on any energy grid.
#include <cmath>
#include <vector>

#include "common.cuh"

using namespace leo2d;

namespace {

__device__ __forceinline__ double jackson(int P, int i) {
  const double pi = 3.141592653589793;
  return ((P - i) * cos((pi * i) / P) + sin((pi * i) / P) / tan(pi / P)) / (P);
}

__global__ void k_mean_jackson(const double* __restrict__ mu, int P, int sets, double* __restrict__ in) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    double m = 0.0;
    if (sets == 1) {
      m = mu[i];
    } else {
      for (int s = 0; s < sets; ++s) m = m + mu[(size_t)s * P + i] / ((double)sets);
    }
    in[i] = jackson(P, i) * m;
  }
}

__global__ void k_dct3_nodes(const double* __restrict__ in, int P, double rescale, double shift,
                             double scale, double* __restrict__ dos, double* __restrict__ energies) {
  const double pi = 3.141592653589793;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P; k += gridDim.x * blockDim.x) {
    double acc = in[0];
    const int64_t q = 2 * (int64_t)k + 1, den = 2 * (int64_t)P, period = 4 * (int64_t)P;
    for (int j = 1; j < P; ++j) {
      const int64_t num = ((int64_t)j * q) % period;
      acc += 2.0 * in[j] * cospi((double)num / (double)den);
    }
    const double E = shift + rescale * cos((k * 1.0 + 0.5) * pi / P);
    if (energies) energies[k] = E;
    dos[k] = scale * acc / (pi * sqrt(rescale * rescale - (E - shift) * (E - shift)));
  }
}

__global__ void k_reconstruct(const double* __restrict__ g, int P, const double* __restrict__ E,
                              int64_t nE, double rescale, double center, double scale,
                              double* __restrict__ out) {
  const double pi = 3.141592653589793;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nE;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double x = (E[e] - center) / rescale;
    if (!(x > -1.0 && x < 1.0)) {
      out[e] = 0.0;
      continue;
    }
    double t0 = 1.0, t1 = x, acc = g[0];
    if (P > 1) acc += 2.0 * g[1] * t1;
    for (int n = 2; n < P; ++n) {
      const double t2 = 2.0 * x * t1 - t0;
      acc += 2.0 * g[n] * t2;
      t0 = t1;
      t1 = t2;
    }
    out[e] = scale * acc / (pi * rescale * sqrt(1.0 - x * x));
  }
}

}  // namespace

extern "C" {

leo2d_status leo2d_dos_transform(leo2d_ctx* ctx, const double* mu, int32_t poly_order,
                                 int32_t num_sets, double rescale, double shift, double scale,
                                 double* dos_out, double* energies_out) {
  if (!ctx || !mu || !dos_out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_REQUIRE(poly_order >= 2 && num_sets >= 1, "poly_order >= 2 and num_sets >= 1 required");
    LEO_REQUIRE(rescale > 0 && std::isfinite(rescale) && std::isfinite(shift), "bad rescale/shift");
    LEO_CUDA(cudaSetDevice(ctx->device));
    const int P = poly_order;
    DevBuf<double> dmu((size_t)P * num_sets), din(P), ddos(P), dE(P);
    h2d(ctx, dmu.p, mu, (size_t)P * num_sets);
    launch(ctx, "mean_jackson", [&] {
      k_mean_jackson<<<grid_for(P, 256), 256, 0, ctx->stream>>>(dmu.p, P, num_sets, din.p);
    });
    launch(ctx, "dct3_nodes", [&] {
      k_dct3_nodes<<<grid_for(P, 128), 128, 0, ctx->stream>>>(din.p, P, rescale, shift, scale, ddos.p, dE.p);
    });
    d2h(ctx, dos_out, ddos.p, P);
    if (energies_out) d2h(ctx, energies_out, dE.p, P);
    ctx_sync(ctx);
  });
}

leo2d_status leo2d_dos_reconstruct(leo2d_ctx* ctx, const double* mu, int32_t poly_order,
                                   const double* energies, int64_t num_energies, double rescale,
                                   double center, double scale, double* dos_out) {
  if (!ctx || !mu || !energies || !dos_out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_REQUIRE(poly_order >= 2 && num_energies >= 0, "bad sizes");
    LEO_REQUIRE(rescale > 0 && std::isfinite(rescale) && std::isfinite(center), "bad rescale/center");
    LEO_CUDA(cudaSetDevice(ctx->device));
    const int P = poly_order;
    DevBuf<double> dmu(P), dg(P), dE(std::max<int64_t>(num_energies, 1)),
        dout(std::max<int64_t>(num_energies, 1));
    h2d(ctx, dmu.p, mu, P);
    h2d(ctx, dE.p, energies, num_energies);
    launch(ctx, "mean_jackson", [&] {
      k_mean_jackson<<<grid_for(P, 256), 256, 0, ctx->stream>>>(dmu.p, P, 1, dg.p);
    });
    if (num_energies > 0)
      launch(ctx, "reconstruct", [&] {
        k_reconstruct<<<grid_for(num_energies, 128), 128, 0, ctx->stream>>>(dg.p, P, dE.p, num_energies,
                                                                           rescale, center, scale, dout.p);
      });
    d2h(ctx, dos_out, dout.p, num_energies);
    ctx_sync(ctx);
  });
}

}  // extern "C"
