// geom_prepare.cpp - host-side completion of a job's geometry.
//
// Lattices of the two graphene models (src/materials/graphene.h:77-85) and, for
// periodic jobs, Locality::setupSupercell type 1 (src/locality.cpp:153-293):
// twist theta = acos((N^2 + 4NM + M^2) / (2 (N^2 + NM + M^2))) (negated when
// M < N), sheet 0 at angle 0 with supercell strides (N, M; -M, M+N), sheet 1 at
// theta with (M, N; -N, M+N), supercell vectors = strides x lattice; or type 3
// for a helical trilayer (src/locality.cpp:401-532): sheets at -theta, 0, theta
// with the strides of leo2d_geom.trilayer_supercell. Compiled with
// -ffp-contract=off so every value equals the reference's.
#include <cmath>
#include <cstring>

#include "../../include/leo2d_gpu.h"

namespace {

void lattice(int model, double lat[2][2]) {
  const double a = model == LEO2D_MODEL_SIMPLE ? 2.46 : 2.4768;
  lat[0][0] = 1. * a;
  lat[0][1] = 0.;
  lat[1][0] = .5 * a;
  lat[1][1] = 0.866025403784438646764 * a;
}

}  // namespace

extern "C" leo2d_status leo2d_geom_prepare(leo2d_geom* g) {
  if (!g) return LEO2D_ERR_BAD_ARG;
  if (g->num_sheets < 1 || g->num_sheets > LEO2D_MAX_SHEETS) return LEO2D_ERR_BAD_ARG;
  if (g->model != LEO2D_MODEL_REF && g->model != LEO2D_MODEL_SIMPLE) return LEO2D_ERR_BAD_ARG;
  for (int s = 0; s < g->num_sheets; ++s) lattice(g->model, g->lattice[s]);
  if (g->boundary_condition == 1) {
    const int M = g->supercell_m, N = g->supercell_n;
    if (M < 0 || N < 0 || (M == 0 && N == 0)) return LEO2D_ERR_BAD_ARG;
    const bool tri = g->trilayer_supercell != 0;
    if (tri && g->num_sheets != 3) return LEO2D_ERR_BAD_ARG;
    double theta = std::acos((N * N + 4 * N * M + M * M) / (2.0 * (N * N + N * M + M * M)));
    if (M < N) theta = -theta;
    const double h_fac = 1.0;
    for (int i = 0; i < g->num_sheets; ++i) {
      const int group = tri ? i : (i == 0 ? 0 : 1);
      int A1_a1, A1_a2, A2_a1, A2_a2;
      if (tri) {
        const int q = M * M + M * N + N * N;
        if (group == 0) {
          g->angles[i] = -theta;
          A1_a1 = N * N - M * M; A1_a2 = M * M + 2 * M * N; A2_a1 = -(M * M + 2 * M * N); A2_a2 = N * N + 2 * M * N;
        } else if (group == 1) {
          g->angles[i] = 0;
          A1_a1 = 0; A1_a2 = q; A2_a1 = -q; A2_a2 = q;
        } else {
          g->angles[i] = theta;
          A1_a1 = M * M - N * N; A1_a2 = N * N + 2 * M * N; A2_a1 = -(N * N + 2 * M * N); A2_a2 = M * M + 2 * M * N;
        }
      } else if (group == 0) {
        g->angles[i] = 0;
        A1_a1 = N; A1_a2 = M; A2_a1 = -M; A2_a2 = (M + N);
      } else {
        g->angles[i] = theta;
        A1_a1 = h_fac * M; A1_a2 = h_fac * N; A2_a1 = -h_fac * N; A2_a2 = h_fac * (M + N);
      }
      double base[2][2], uc[2][2];
      lattice(g->model, base);
      const double th = 0.0;
      uc[0][0] = std::cos(th) * base[0][0] - std::sin(th) * base[0][1];
      uc[0][1] = std::sin(th) * base[0][0] + std::cos(th) * base[0][1];
      uc[1][0] = std::cos(th) * base[1][0] - std::sin(th) * base[1][1];
      uc[1][1] = std::sin(th) * base[1][0] + std::cos(th) * base[1][1];
      double (*sc)[2] = g->sheet_supercell[i];
      sc[0][0] = A1_a1 * uc[0][0] + A1_a2 * uc[1][0];
      sc[0][1] = A1_a1 * uc[0][1] + A1_a2 * uc[1][1];
      sc[1][0] = A2_a1 * uc[0][0] + A2_a2 * uc[1][0];
      sc[1][1] = A2_a1 * uc[0][1] + A2_a2 * uc[1][1];
      g->sheet_sc_stride[i][0][0] = A1_a1;
      g->sheet_sc_stride[i][0][1] = A1_a2;
      g->sheet_sc_stride[i][1][0] = A2_a1;
      g->sheet_sc_stride[i][1][1] = A2_a2;
      if (i == 0) std::memcpy(g->supercell, sc, sizeof(g->supercell));
    }
  }
  g->prepared = 1;
  return LEO2D_OK;
}
