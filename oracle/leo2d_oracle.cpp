/*
 * leo2d_oracle.cpp - CPU restatement of LEO2D's KPM path (see leo2d_oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library, never shipped in
 * it. Compile with -ffp-contract=off so no multiply-add is fused: the
 * reference's x86-64 build evaluates every product and sum separately, and the
 * bit-exact geometry depends on it.
 */
#include "leo2d_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

namespace {

// tools/numbers.h:43-93
const double kPi = 3.14159265358979323846;
const double kPi_6 = 0.523598775598298873077;
const double kSqrt3_2 = 0.866025403784438646764;
const double kSqrt3_6 = 0.288675134594812882255;

// ---------------------------------------------------------------- materials

// Graphene::a (graphene.h:78); the simple model uses a = 2.46 A.
double lattice_const(int model) { return model == LEO2D_MODEL_SIMPLE ? 2.46 : 2.4768; }

// Graphene::lattice / atom_pos (graphene.h:79-85)
void material_lattice(int model, double lat[2][2], double atom[2][3]) {
  const double a = lattice_const(model);
  lat[0][0] = 1. * a;
  lat[0][1] = 0.;
  lat[1][0] = .5 * a;
  lat[1][1] = kSqrt3_2 * a;
  atom[0][0] = 0.; atom[0][1] = 0.; atom[0][2] = 0.;
  atom[1][0] = 0.5 * a; atom[1][1] = kSqrt3_6 * a; atom[1][2] = 0;
}

// Coupling::Intralayer::graphene (graphene.cpp:13-89): hexagonal homogeneous
// coordinates, shell index r, 9-entry table.
double intralayer(int model, int orow, int ocol, int d0, int d1) {
  int h0 = 2 * d0 + d1;
  int h1 = -1 * d0 + d1;
  if (ocol == 0 && orow == 1) h0 -= 1;
  else if (ocol == 1 && orow == 0) h0 += 1;
  const int r = h0 * (h0 + h1) + h1 * h1;
  if (model == LEO2D_MODEL_SIMPLE) return r == 1 ? -2.7 : 0.0;
  const double t_arr[9] = {0.3504, -2.8922, 0.2425, -0.2656, 0.0235, 0.0524, -0.0209, -0.0148, -0.0211};
  switch (r) {
    case 0: return t_arr[0];
    case 1: return t_arr[1];
    case 3: return t_arr[2];
    case 4: return t_arr[3];
    case 7: return t_arr[4];
    case 9: return t_arr[5];
    case 12: return t_arr[6];
    case 13: return t_arr[7];
    case 16: return t_arr[8];
    default: return 0.;
  }
}

// Coupling::Interlayer::C_to_C (graphene.cpp:91-222). The reference's
// abs(vector[2]) at graphene.cpp:117 binds to the int overload, so the
// decoupling test is |trunc(z)| > 5. The fitted coefficients and the order of
// every operation are kept as in the reference so results agree bit for bit.
double c_to_c(int orow, int ocol, double v0, double v1, double v2, double theta_row,
              double theta_col) {
  if (std::abs((int)v2) > 5) return 0;
  double r = std::sqrt(v0 * v0 + v1 * v1);
  if (r < 8.0) {
    double ac = std::atan2(v1, v0);
    double theta21 = ac - theta_row;
    if (orow == 1) theta21 += kPi_6; else theta21 -= kPi_6;
    double theta12 = ac - theta_col + kPi;
    if (ocol == 1) theta12 += kPi_6; else theta12 -= kPi_6;
    double rs = r / 2.4768;
    double z_eq = 3.35;
    double z_eps = (std::fabs(v2) - z_eq) / z_eq;
    double lambda_0 = 0.310 - 1.882 * z_eps + 7.741 * z_eps * z_eps;
    double xi_0 = 1.750 - 1.618 * z_eps + 1.848 * z_eps * z_eps;
    double kappa_0 = 1.990 + 1.007 * z_eps + 2.427 * z_eps * z_eps;
    double lambda_3 = -0.068 + 0.399 * z_eps - 1.739 * z_eps * z_eps;
    double xi_3 = 3.286 - 0.914 * z_eps + 12.011 * z_eps * z_eps;
    double x_3 = 0.500 + 0.322 * z_eps + 0.908 * z_eps * z_eps;
    double lambda_6 = -0.008 + 0.046 * z_eps - 0.183 * z_eps * z_eps;
    double xi_6 = 2.272 - 0.721 * z_eps - 4.414 * z_eps * z_eps;
    double x_6 = 1.217 + 0.027 * z_eps - 0.658 * z_eps * z_eps;
    double kappa_6 = 1.562 - 0.371 * z_eps - 0.134 * z_eps * z_eps;
    double V0 = lambda_0 * std::exp(-xi_0 * (rs) * (rs)) * std::cos(kappa_0 * rs);
    double V3 = lambda_3 * rs * rs * std::exp(-xi_3 * (rs - x_3) * (rs - x_3));
    double V6 = lambda_6 * std::exp(-xi_6 * (rs - x_6) * (rs - x_6)) * std::sin(kappa_6 * rs);
    double t = V0 + V3 * (std::cos(3 * theta12) + std::cos(3 * theta21)) +
               V6 * (std::cos(6 * theta12) + std::cos(6 * theta21));
    double d = 8.0 - r;
    if (d < 1. && d > 0.) t *= std::exp(1. - 1. / (d * d));
    return t;
  }
  return 0.;
}

// Simple interlayer model, already divided by the energy rescale:
// (0.33 / rescale) exp(-(r - 3.35) / 0.45) for the 3-D distance r < 8 A, with
// the quotients taken as products by (0.33 / rescale) and by the FP64 value of
// 1 / 0.45 (the form the device assembly evaluates).
double simple_inter_t(double v0, double v1, double v2, double rescale) {
  const double inv_decay = 1.0 / 0.45;
  const double amp = 0.33 / rescale;
  double r = std::sqrt(v0 * v0 + v1 * v1 + v2 * v2);
  if (r < 8.0) return amp * std::exp(-(r - 3.35) * inv_decay);
  return 0.0;
}

// Interlayer hopping divided by the energy rescale (generateRealH's t / energy_rescale).
double interlayer_t(int model, int orow, int ocol, double v0, double v1, double v2, double th_row,
                    double th_col, double rescale) {
  if (model == LEO2D_MODEL_SIMPLE) return simple_inter_t(v0, v1, v2, rescale);
  return c_to_c(orow, ocol, v0, v1, v2, th_row, th_col) / rescale;
}

// ---------------------------------------------------------------- sheets

struct SheetGeo {
  int min0, min1, max0, max1;
  int H, W, n_orb;
  double max_R;
  int bc;
  double a[2][2], atom[2][3], a_inv[2][2];
  double sc[2][2], sc_inv[2][2];
  int stride[2][2];
  std::vector<int32_t> grid;  // [H][W][n_orb] -> local index or -1
  std::vector<int32_t> idx;   // [k][3] = (i, j, l)
  int max_index = 0;

  // Sheet::posAtomGrid (sheet.cpp:482-531), real space, no global shifts
  void pos_grid(int i, int j, int l, double p[3]) const {
    int ii = i + min0, jj = j + min1;
    p[0] = ii * a[0][0] + jj * a[1][0] + atom[l][0];
    p[1] = ii * a[0][1] + jj * a[1][1] + atom[l][1];
    p[2] = atom[l][2];
  }
  // Sheet::checkShape (sheet.cpp:537-559)
  bool check_shape(const double p[3]) const {
    if (bc == 1) {
      double delta = 0.0, grid_delta = 0.000001;
      double i = (p[0] + delta) * sc_inv[0][0] + (p[1] + delta) * sc_inv[0][1];
      double j = (p[0] + delta) * sc_inv[1][0] + (p[1] + delta) * sc_inv[1][1];
      return i >= 0.0 - grid_delta && i < 1.0 - grid_delta && j >= 0.0 - grid_delta &&
             j < 1.0 - grid_delta;
    }
    return std::pow(p[0], 2) + std::pow(p[1], 2) < std::pow(max_R, 2);
  }
  // Sheet::gridToIndex (sheet.cpp:572-583)
  int grid_to_index(int i, int j, int l) const {
    if (i >= 0 && i < H && j >= 0 && j < W && l >= 0 && l < n_orb)
      return grid[((size_t)i * W + j) * n_orb + l];
    return -1;
  }
  // Sheet::findNearest (sheet.cpp:856-883)
  int find_nearest(const double p[3], int dim) const {
    if (dim == 0) {
      double i_new = a_inv[0][0] * p[0] + a_inv[0][1] * p[1];
      return std::min(std::max(int(std::floor(i_new)), min0), max0) - min0;
    }
    double j_new = a_inv[1][0] * p[0] + a_inv[1][1] * p[1];
    return std::min(std::max(int(std::floor(j_new)), min1), max1) - min1;
  }
};

void make_sheet(const leo2d_geom* g, int s, SheetGeo& sh) {
  sh.min0 = g->min_shape[s][0];
  sh.min1 = g->min_shape[s][1];
  sh.max0 = g->max_shape[s][0];
  sh.max1 = g->max_shape[s][1];
  sh.H = sh.max0 - sh.min0;
  sh.W = sh.max1 - sh.min1;
  sh.n_orb = 2;
  sh.max_R = g->max_R[s];
  sh.bc = g->boundary_condition;
  double atom[2][3];
  material_lattice(g->model, sh.a, atom);
  std::memcpy(sh.atom, atom, sizeof(atom));
  // Sheet::setInverse (sheet.cpp:888-908)
  double a11 = sh.a[0][0], a12 = sh.a[0][1], a21 = sh.a[1][0], a22 = sh.a[1][1];
  double det_a = a11 * a22 - a12 * a21;
  sh.a_inv[0][0] = a22 / det_a;
  sh.a_inv[0][1] = -a21 / det_a;
  sh.a_inv[1][0] = -a12 / det_a;
  sh.a_inv[1][1] = a11 / det_a;
  if (sh.bc == 1) {
    // Sheet::setSupercell (sheet.cpp:910-928)
    for (int x = 0; x < 2; ++x)
      for (int y = 0; y < 2; ++y) {
        sh.sc[x][y] = g->sheet_supercell[s][x][y];
        sh.stride[x][y] = g->sheet_sc_stride[s][x][y];
      }
    double det = sh.sc[0][0] * sh.sc[1][1] - sh.sc[0][1] * sh.sc[1][0];
    sh.sc_inv[0][0] = sh.sc[1][1] / det;
    sh.sc_inv[0][1] = -sh.sc[1][0] / det;
    sh.sc_inv[1][0] = -sh.sc[0][1] / det;
    sh.sc_inv[1][1] = sh.sc[0][0] / det;
  }
  // Sheet::setIndex (sheet.cpp:217-285)
  sh.grid.assign((size_t)sh.H * sh.W * sh.n_orb, -1);
  int k = 0;
  for (int i = 0; i < sh.H; ++i)
    for (int j = 0; j < sh.W; ++j)
      for (int l = 0; l < sh.n_orb; ++l) {
        double p[3];
        sh.pos_grid(i, j, l, p);
        if (sh.check_shape(p)) {
          sh.grid[((size_t)i * sh.W + j) * sh.n_orb + l] = k;
          sh.idx.push_back(i);
          sh.idx.push_back(j);
          sh.idx.push_back(l);
          ++k;
        }
      }
  sh.max_index = k;
}

struct Pair {
  int32_t i, j;
  double t;
  int32_t sc0, sc1;
};

}  // namespace

struct oracle_h {
  leo2d_geom g;
  int64_t n = 0;
  std::vector<int32_t> grid4;  // [n][4]
  std::vector<double> index_to_pos, i2pos;
  std::vector<Pair> intra, inter;
  std::vector<int64_t> rowptr;
  std::vector<int32_t> col;
  std::vector<double> val, dx, dy;
  std::vector<int64_t> sheet_base;
  std::vector<SheetGeo> sheets;
};

extern "C" {

// Locality::setupSupercell, type 1 (locality.cpp:153-293) and type 3, the
// helical trilayer (locality.cpp:401-532), + lattices.
int oracle_geom_prepare(leo2d_geom* g) {
  if (!g || g->num_sheets < 1 || g->num_sheets > LEO2D_MAX_SHEETS) return 1;
  for (int s = 0; s < g->num_sheets; ++s) {
    double atom[2][3];
    material_lattice(g->model, g->lattice[s], atom);
  }
  if (g->boundary_condition == 1) {
    const int M = g->supercell_m, N = g->supercell_n;
    double theta = std::acos((N * N + 4 * N * M + M * M) / (2.0 * (N * N + N * M + M * M)));
    if (M < N) theta = -theta;
    double h_fac = 1.0;
    const int type = g->trilayer_supercell ? 3 : 1;
    if (type == 3 && g->num_sheets != 3) return 1;
    for (int i = 0; i < g->num_sheets; ++i) {
      // sc_groups: {0, 1} for a bilayer (locality.cpp:156-160), {0, 1, 2} for
      // the trilayer (locality.cpp:404-409)
      const int group = type == 3 ? i : (i < 2 ? i : 1);
      int A1_a1, A1_a2, A2_a1, A2_a2;
      if (type == 3) {
        if (group == 0) {
          g->angles[i] = -theta;
          A1_a1 = std::pow(N, 2) - std::pow(M, 2);
          A1_a2 = std::pow(M, 2) + 2 * M * N;
          A2_a1 = -(std::pow(M, 2) + 2 * M * N);
          A2_a2 = std::pow(N, 2) + 2 * M * N;
        } else if (group == 1) {
          g->angles[i] = 0;
          A1_a1 = 0;
          A1_a2 = std::pow(M, 2) + (M * N) + std::pow(N, 2);
          A2_a1 = -(std::pow(N, 2) + (M * N) + std::pow(M, 2));
          A2_a2 = std::pow(N, 2) + M * N + std::pow(M, 2);
        } else {
          g->angles[i] = theta;
          A1_a1 = std::pow(M, 2) - std::pow(N, 2);
          A1_a2 = std::pow(N, 2) + 2 * M * N;
          A2_a1 = -(std::pow(N, 2) + (2 * M * N));
          A2_a2 = std::pow(M, 2) + (2 * M * N);
        }
      } else if (group == 0) {
        g->angles[i] = 0;
        A1_a1 = N; A1_a2 = M; A2_a1 = -M; A2_a2 = (M + N);
      } else {
        g->angles[i] = theta;
        A1_a1 = h_fac * M; A1_a2 = h_fac * N; A2_a1 = -h_fac * N; A2_a2 = h_fac * (M + N);
      }
      double base[2][2], atom[2][3];
      material_lattice(g->model, base, atom);
      double th = 0.0, uc[2][2];
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
  return 0;
}

int oracle_build(const leo2d_geom* gin, oracle_h** out) {
  if (!gin || !out || !gin->prepared) return 1;
  oracle_h* h = new oracle_h();
  h->g = *gin;
  const leo2d_geom& g = h->g;
  const int S = g.num_sheets;
  h->sheets.resize(S);
  for (int s = 0; s < S; ++s) make_sheet(&g, s, h->sheets[s]);

  // Hstruct::setIndex (hstruct.cpp:69-110)
  int64_t n = 0;
  for (int s = 0; s < S; ++s) {
    h->sheet_base.push_back(n);
    n += h->sheets[s].max_index;
  }
  h->n = n;
  h->grid4.resize(4 * (size_t)n);
  for (int s = 0; s < S; ++s)
    for (int k = 0; k < h->sheets[s].max_index; ++k) {
      int64_t gk = h->sheet_base[s] + k;
      for (int d = 0; d < 3; ++d) h->grid4[4 * gk + d] = h->sheets[s].idx[3 * (size_t)k + d];
      h->grid4[4 * gk + 3] = s;
    }

  // Hstruct::posAtomIndex (hstruct.cpp:150-218) with zero sheet shifts.
  auto pos_index = [&](int64_t k, double p[3]) {
    int s = h->grid4[4 * k + 3];
    const SheetGeo& sh = h->sheets[s];
    double lp[3];
    sh.pos_grid(h->grid4[4 * k], h->grid4[4 * k + 1], h->grid4[4 * k + 2], lp);
    double theta = g.angles[s];
    double z0 = 0;
    p[0] = lp[0] * std::cos(theta) - lp[1] * std::sin(theta) + z0 * sh.a[0][0] + z0 * sh.a[1][0];
    p[1] = lp[0] * std::sin(theta) + lp[1] * std::cos(theta) + z0 * sh.a[0][1] + z0 * sh.a[1][1];
    p[2] = lp[2] + g.heights[s];
  };
  h->index_to_pos.resize(3 * (size_t)n);
  for (int64_t k = 0; k < n; ++k) pos_index(k, &h->index_to_pos[3 * k]);

  // Hstruct::findNearest (hstruct.cpp:224-288), zero shifts.
  auto hfind = [&](const double p[3], int s, int dim) {
    const SheetGeo& sh = h->sheets[s];
    double theta = -g.angles[s];
    double z0 = 0;
    double x_new = p[0] * std::cos(theta) - p[1] * std::sin(theta) + z0 * sh.a[0][0] + z0 * sh.a[1][0];
    double y_new = p[0] * std::sin(theta) + p[1] * std::cos(theta) + z0 * sh.a[0][1] + z0 * sh.a[1][1];
    if (dim == 0) {
      double i_new = sh.a_inv[0][0] * x_new + sh.a_inv[0][1] * y_new;
      return std::min(std::max(int(std::floor(i_new)), sh.min0), sh.max0) - sh.min0;
    }
    double j_new = sh.a_inv[1][0] * x_new + sh.a_inv[1][1] * y_new;
    return std::min(std::max(int(std::floor(j_new)), sh.min1), sh.max1) - sh.min1;
  };

  const int sc_stride = g.boundary_condition == 1 ? g.sc_search_size : 0;
  auto by_col = [](const Pair& a, const Pair& b) { return a.j < b.j; };

  // Hstruct::getInterPairs (hstruct.cpp:298-632): sheet below, then above;
  // window +-6 cells clipped to the grid; keep in-plane distance < 12.5 A.
  {
    const int searchsize = 6;
    const double inter_cutoff = 12.5;
    for (int64_t kh = 0; kh < n; ++kh) {
      std::vector<Pair> kp;
      const int sh = h->grid4[4 * kh + 3];
      double khp[3];
      pos_index(kh, khp);
      for (int dxs = -sc_stride; dxs < sc_stride + 1; ++dxs)
        for (int dys = -sc_stride; dys < sc_stride + 1; ++dys) {
          double sc_disp0 = 0.0, sc_disp1 = 0.0;
          int sc0 = 0, sc1 = 0;
          if (g.boundary_condition == 1) {
            sc0 = dxs; sc1 = dys;
            sc_disp0 = dxs * g.supercell[0][0] + dys * g.supercell[1][0];
            sc_disp1 = dxs * g.supercell[0][1] + dys * g.supercell[1][1];
          }
          double ph[3] = {khp[0] + sc_disp0, khp[1] + sc_disp1, khp[2]};
          for (int side = 0; side < 2; ++side) {
            int s0 = side == 0 ? sh - 1 : sh + 1;
            if (s0 < 0 || s0 >= S) continue;
            int i0 = hfind(ph, s0, 0), j0 = hfind(ph, s0, 1);
            const SheetGeo& o = h->sheets[s0];
            int64_t base = h->sheet_base[s0];
            for (int i = std::max(0, i0 - searchsize); i < std::min(o.H, i0 + searchsize); ++i)
              for (int j = std::max(0, j0 - searchsize); j < std::min(o.W, j0 + searchsize); ++j)
                for (int l = 0; l < o.n_orb; ++l) {
                  int k2 = o.grid_to_index(i, j, l);
                  if (k2 == -1) continue;
                  double p2[3];
                  pos_index(k2 + base, p2);
                  double x2 = p2[0], y2 = p2[1];
                  if ((x2 - ph[0]) * (x2 - ph[0]) + (y2 - ph[1]) * (y2 - ph[1]) <
                      inter_cutoff * inter_cutoff)
                    kp.push_back(Pair{(int32_t)kh, (int32_t)(k2 + base), 0.0, sc0, sc1});
                }
          }
        }
      if (g.boundary_condition == 1) std::stable_sort(kp.begin(), kp.end(), by_col);
      h->inter.insert(h->inter.end(), kp.begin(), kp.end());
    }
  }

  // Hstruct::getIntraPairs -> Sheet::getIntraPairs (sheet.cpp:624-752): window
  // [i0-4, i0+4) x [j0-4, j0+4) in the sheet's own frame; keep t != 0 or the
  // home image.
  {
    const int searchsize = 4;
    for (int s = 0; s < S; ++s) {
      const SheetGeo& sh = h->sheets[s];
      const int64_t start = h->sheet_base[s];
      for (int kh = 0; kh < sh.max_index; ++kh) {
        std::vector<Pair> kp;
        const int ih = sh.idx[3 * (size_t)kh], jh = sh.idx[3 * (size_t)kh + 1];
        const int l0 = sh.idx[3 * (size_t)kh + 2];
        double khp[3];
        sh.pos_grid(ih, jh, l0, khp);
        for (int dxs = -sc_stride; dxs < sc_stride + 1; ++dxs)
          for (int dys = -sc_stride; dys < sc_stride + 1; ++dys) {
            double sc_disp0 = 0.0, sc_disp1 = 0.0;
            int sc0 = 0, sc1 = 0;
            if (g.boundary_condition == 1) {
              sc0 = dxs; sc1 = dys;
              sc_disp0 = dxs * sh.sc[0][0] + dys * sh.sc[1][0];
              sc_disp1 = dxs * sh.sc[0][1] + dys * sh.sc[1][1];
            }
            double ph[3] = {khp[0] + sc_disp0, khp[1] + sc_disp1, khp[2]};
            int i0 = sh.find_nearest(ph, 0), j0 = sh.find_nearest(ph, 1);
            for (int i = i0 - searchsize; i < i0 + searchsize; ++i)
              for (int j = j0 - searchsize; j < j0 + searchsize; ++j)
                for (int l = 0; l < sh.n_orb; ++l) {
                  int k2 = sh.grid_to_index(i, j, l);
                  if (k2 == -1) continue;
                  int gd0 = i - ih, gd1 = j - jh;
                  if (g.boundary_condition == 1) {
                    gd0 = gd0 - dxs * sh.stride[0][0] - dys * sh.stride[1][0];
                    gd1 = gd1 - dxs * sh.stride[0][1] - dys * sh.stride[1][1];
                  }
                  double t = intralayer(g.model, l0, l, gd0, gd1);
                  if (t != 0 || (dxs == 0 && dys == 0))
                    kp.push_back(Pair{(int32_t)(kh + start), (int32_t)(k2 + start), t, sc0, sc1});
                }
          }
        if (g.boundary_condition == 1) std::stable_sort(kp.begin(), kp.end(), by_col);
        h->intra.insert(h->intra.end(), kp.begin(), kp.end());
      }
    }
  }

  // Locality::setConfigPositions (locality.cpp:3618-3642), zero shifts.
  h->i2pos.resize(3 * (size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    int s = h->grid4[4 * i + 3];
    const SheetGeo& sh = h->sheets[s];
    double theta = g.angles[s], s1a[2][2];
    for (int d = 0; d < 2; ++d) {
      s1a[d][0] = std::cos(theta) * sh.a[d][0] - std::sin(theta) * sh.a[d][1];
      s1a[d][1] = std::sin(theta) * sh.a[d][0] + std::cos(theta) * sh.a[d][1];
    }
    // the job's sheet shifts (Job_params "shifts"; zero unless set)
    const double sh0 = g.shifts[s][0], sh1 = g.shifts[s][1];
    h->i2pos[3 * i + 0] = h->index_to_pos[3 * i + 0] + sh0 * s1a[0][0] + sh1 * s1a[1][0];
    h->i2pos[3 * i + 1] = h->index_to_pos[3 * i + 1] + sh0 * s1a[0][1] + sh1 * s1a[1][1];
    h->i2pos[3 * i + 2] = h->index_to_pos[3 * i + 2];
  }

  // Locality::generateRealH (locality.cpp:3900-4321)
  const double rescale = g.energy_rescale, shift = g.energy_shift;
  const size_t n_intra = h->intra.size(), n_inter = h->inter.size();
  const size_t max_nnz = n_intra + n_inter;
  h->val.assign(max_nnz, 0.0);
  h->dx.assign(max_nnz, 0.0);
  h->dy.assign(max_nnz, 0.0);
  h->col.assign(max_nnz, 0);
  h->rowptr.assign(n + 1, 0);
  size_t ic = 0, ec = 0, cnt = 0;
  const double* P = h->i2pos.data();
  for (int64_t ki = 0; ki < n; ++ki) {
    h->rowptr[ki] = (int64_t)cnt;
    while (ic < n_intra && h->intra[ic].i == ki) {
      const Pair& pr = h->intra[ic];
      int64_t nk = pr.j;
      double shx = 0.0, shy = 0.0;
      if (g.boundary_condition == 1) {
        shx = pr.sc0 * g.supercell[0][0] + pr.sc1 * g.supercell[1][0];
        shy = pr.sc0 * g.supercell[0][1] + pr.sc1 * g.supercell[1][1];
      }
      double x1 = P[3 * ki] + shx, y1 = P[3 * ki + 1] + shy;
      double x2 = P[3 * nk], y2 = P[3 * nk + 1];
      // (the diagonal: generateRealH's onSiteE term z E with USE_E_FIELD)
      double t = nk == ki ? (g.e_field != 0.0 ? (pr.t + shift + P[3 * ki + 2] * g.e_field) / rescale
                                              : (pr.t + shift) / rescale)
                          : pr.t / rescale;
      if (t != 0) {
        h->val[cnt] += t;
        h->dx[cnt] += (x1 - x2) * t;
        h->dy[cnt] += (y1 - y2) * t;
      }
      if (ic + 1 == n_intra || h->intra[ic + 1].i != ki || h->intra[ic + 1].j != nk) {
        h->col[cnt] = (int32_t)nk;
        ++cnt;
      }
      ++ic;
    }
    while (ec < n_inter && h->inter[ec].i == ki) {
      const Pair& pr = h->inter[ec];
      int64_t nk = pr.j;
      double shx = 0.0, shy = 0.0;
      if (g.boundary_condition == 1) {
        shx = pr.sc0 * g.supercell[0][0] + pr.sc1 * g.supercell[1][0];
        shy = pr.sc0 * g.supercell[0][1] + pr.sc1 * g.supercell[1][1];
      }
      double x1 = P[3 * ki] + shx, y1 = P[3 * ki + 1] + shy, z1 = P[3 * ki + 2];
      double x2 = P[3 * nk], y2 = P[3 * nk + 1], z2 = P[3 * nk + 2];
      int o1 = h->grid4[4 * ki + 2], o2 = h->grid4[4 * nk + 2];
      double th1 = g.angles[h->grid4[4 * ki + 3]], th2 = g.angles[h->grid4[4 * nk + 3]];
      double t = interlayer_t(g.model, o1, o2, x2 - x1, y2 - y1, z2 - z1, th1, th2, rescale);
      if (t != 0) {
        h->val[cnt] += t;
        h->dx[cnt] += (x1 - x2) * t;
        h->dy[cnt] += (y1 - y2) * t;
      }
      if (ec + 1 == n_inter || h->inter[ec + 1].i != ki || h->inter[ec + 1].j != nk) {
        h->col[cnt] = (int32_t)nk;
        ++cnt;
      }
      ++ec;
    }
  }
  h->rowptr[n] = (int64_t)cnt;
  h->col.resize(cnt);
  h->val.resize(cnt);
  h->dx.resize(cnt);
  h->dy.resize(cnt);
  *out = h;
  return 0;
}

void oracle_bloch(const oracle_h* h, double kx, double ky, double* re, double* im) {
  const leo2d_geom& g = h->g;
  const int64_t n = h->n;
  const double rescale = g.energy_rescale, shift = g.energy_shift;
  const double* P = h->i2pos.data();
  const size_t n_intra = h->intra.size(), n_inter = h->inter.size();
  std::vector<std::complex<double>> v(h->col.size(), std::complex<double>(0.0));
  size_t ic = 0, ec = 0, cnt = 0;
  // one pair: its value and the image shift of the row (generateCpxH, as generateRealH)
  auto add = [&](const Pair& pr, int64_t ki, double t) {
    double shx = 0.0, shy = 0.0;
    if (g.boundary_condition == 1) {
      shx = pr.sc0 * g.supercell[0][0] + pr.sc1 * g.supercell[1][0];
      shy = pr.sc0 * g.supercell[0][1] + pr.sc1 * g.supercell[1][1];
    }
    const double x1 = P[3 * ki] + shx, y1 = P[3 * ki + 1] + shy;
    const double x2 = P[3 * pr.j], y2 = P[3 * pr.j + 1];
    // Locality::peierlsPhase (locality.cpp:7157-7161), then k.(r2 - r1) (4896-4900)
    double phase = 3.14e-5 * g.b_field * (x2 - x1) * (0.5) * (y1 + y2);
    phase = phase + kx * (x2 - x1) + ky * (y2 - y1);
    const std::complex<double> z = std::polar(t, phase);
    if (z != std::complex<double>(0.0)) v[cnt] += z;
  };
  for (int64_t ki = 0; ki < n; ++ki) {
    while (ic < n_intra && h->intra[ic].i == ki) {
      const Pair& pr = h->intra[ic];
      const bool home = pr.sc0 == 0 && pr.sc1 == 0;
      const double t = (pr.j == ki && home) ? (g.e_field != 0.0 ? (pr.t + shift + P[3 * ki + 2] * g.e_field) / rescale
                                                                 : (pr.t + shift) / rescale)
                                            : pr.t / rescale;
      add(pr, ki, t);
      if (ic + 1 == n_intra || h->intra[ic + 1].i != ki || h->intra[ic + 1].j != pr.j) ++cnt;
      ++ic;
    }
    while (ec < n_inter && h->inter[ec].i == ki) {
      const Pair& pr = h->inter[ec];
      double shx = 0.0, shy = 0.0;
      if (g.boundary_condition == 1) {
        shx = pr.sc0 * g.supercell[0][0] + pr.sc1 * g.supercell[1][0];
        shy = pr.sc0 * g.supercell[0][1] + pr.sc1 * g.supercell[1][1];
      }
      const double x1 = P[3 * ki] + shx, y1 = P[3 * ki + 1] + shy, z1 = P[3 * ki + 2];
      const double x2 = P[3 * pr.j], y2 = P[3 * pr.j + 1], z2 = P[3 * pr.j + 2];
      const int o1 = h->grid4[4 * ki + 2], o2 = h->grid4[4 * pr.j + 2];
      const double th1 = g.angles[h->grid4[4 * ki + 3]], th2 = g.angles[h->grid4[4 * pr.j + 3]];
      add(pr, ki, interlayer_t(g.model, o1, o2, x2 - x1, y2 - y1, z2 - z1, th1, th2, rescale));
      if (ec + 1 == n_inter || h->inter[ec + 1].i != ki || h->inter[ec + 1].j != pr.j) ++cnt;
      ++ec;
    }
  }
  for (size_t e = 0; e < v.size(); ++e) {
    re[e] = v[e].real();
    im[e] = v[e].imag();
  }
}

void oracle_free(oracle_h* h) { delete h; }

void oracle_info(const oracle_h* h, int64_t* n, int64_t* nnz, int64_t* n_intra, int64_t* n_inter) {
  if (n) *n = h->n;
  if (nnz) *nnz = h->rowptr.empty() ? 0 : h->rowptr[h->n];
  if (n_intra) *n_intra = (int64_t)h->intra.size();
  if (n_inter) *n_inter = (int64_t)h->inter.size();
}

void oracle_get(const oracle_h* h, int64_t* rowptr, int32_t* col, double* val, double* val_dx,
                double* val_dy, int32_t* index_to_grid, double* pos) {
  const size_t nnz = h->col.size();
  if (rowptr) std::memcpy(rowptr, h->rowptr.data(), (h->n + 1) * sizeof(int64_t));
  if (col) std::memcpy(col, h->col.data(), nnz * sizeof(int32_t));
  if (val) std::memcpy(val, h->val.data(), nnz * sizeof(double));
  if (val_dx) std::memcpy(val_dx, h->dx.data(), nnz * sizeof(double));
  if (val_dy) std::memcpy(val_dy, h->dy.data(), nnz * sizeof(double));
  if (index_to_grid) std::memcpy(index_to_grid, h->grid4.data(), h->grid4.size() * sizeof(int32_t));
  if (pos) std::memcpy(pos, h->i2pos.data(), h->i2pos.size() * sizeof(double));
}

void oracle_get_pairs(const oracle_h* h, int32_t* intra_pairs, double* intra_t, int32_t* intra_sc,
                      int32_t* inter_pairs, int32_t* inter_sc) {
  for (size_t x = 0; x < h->intra.size(); ++x) {
    if (intra_pairs) { intra_pairs[2 * x] = h->intra[x].i; intra_pairs[2 * x + 1] = h->intra[x].j; }
    if (intra_t) intra_t[x] = h->intra[x].t;
    if (intra_sc) { intra_sc[2 * x] = h->intra[x].sc0; intra_sc[2 * x + 1] = h->intra[x].sc1; }
  }
  for (size_t x = 0; x < h->inter.size(); ++x) {
    if (inter_pairs) { inter_pairs[2 * x] = h->inter[x].i; inter_pairs[2 * x + 1] = h->inter[x].j; }
    if (inter_sc) { inter_sc[2 * x] = h->inter[x].sc0; inter_sc[2 * x + 1] = h->inter[x].sc1; }
  }
}

// Hstruct::getShiftConfigs (hstruct.cpp:672-820): for every orbital of a
// bilayer, the fractional offset of its cell's orbital-0 site from the site
// of the other sheet found by Hstruct::findNearest, in that sheet's rotated
// lattice, wrapped to [0,1). Returns 1 unless there are exactly two sheets.
int oracle_shift_configs(const oracle_h* h, double* out) {
  const leo2d_geom& g = h->g;
  if (g.num_sheets != 2) return 1;
  double inv[2][2][2];
  for (int s = 0; s < 2; ++s) {
    const double theta = g.angles[s];
    const SheetGeo& sh = h->sheets[s];
    double u[2][2];
    u[0][0] = std::cos(theta) * sh.a[0][0] - std::sin(theta) * sh.a[0][1];
    u[0][1] = std::sin(theta) * sh.a[0][0] + std::cos(theta) * sh.a[0][1];
    u[1][0] = std::cos(theta) * sh.a[1][0] - std::sin(theta) * sh.a[1][1];
    u[1][1] = std::sin(theta) * sh.a[1][0] + std::cos(theta) * sh.a[1][1];
    const double det = u[0][0] * u[1][1] - u[0][1] * u[1][0];
    inv[s][0][0] = u[1][1] / det;
    inv[s][0][1] = -u[1][0] / det;
    inv[s][1][0] = -u[0][1] / det;
    inv[s][1][1] = u[0][0] / det;
  }
  // Hstruct::findNearest (hstruct.cpp:224-288), solver_space 0, zero shifts
  auto hfind = [&](const double p[3], int s, int dim) {
    const SheetGeo& sh = h->sheets[s];
    const double theta = -g.angles[s];
    const double z0 = 0;
    const double x_new = p[0] * std::cos(theta) - p[1] * std::sin(theta) + z0 * sh.a[0][0] + z0 * sh.a[1][0];
    const double y_new = p[0] * std::sin(theta) + p[1] * std::cos(theta) + z0 * sh.a[0][1] + z0 * sh.a[1][1];
    if (dim == 0) {
      const double i_new = sh.a_inv[0][0] * x_new + sh.a_inv[0][1] * y_new;
      return std::min(std::max(int(std::floor(i_new)), sh.min0), sh.max0) - sh.min0;
    }
    const double j_new = sh.a_inv[1][0] * x_new + sh.a_inv[1][1] * y_new;
    return std::min(std::max(int(std::floor(j_new)), sh.min1), sh.max1) - sh.min1;
  };
  for (int64_t k = 0; k < h->n; ++k) {
    const int s_here = h->grid4[4 * k + 3];
    const int s = s_here == 0 ? 1 : 0;
    double orig[3];
    h->sheets[s_here].pos_grid(h->grid4[4 * k], h->grid4[4 * k + 1], 0, orig);
    const double th = g.angles[s_here];
    double here[3];
    here[0] = std::cos(th) * orig[0] - std::sin(th) * orig[1];
    here[1] = std::sin(th) * orig[0] + std::cos(th) * orig[1];
    here[2] = 0;
    const int ni = hfind(here, s, 0), nj = hfind(here, s, 1);
    double sp[3];
    h->sheets[s].pos_grid(ni, nj, 0, sp);
    const double ts = g.angles[s];
    const double np0 = std::cos(ts) * sp[0] - std::sin(ts) * sp[1];
    const double np1 = std::sin(ts) * sp[0] + std::cos(ts) * sp[1];
    const double cr0 = here[0] - np0, cr1 = here[1] - np1;
    double c0 = cr0 * inv[s][0][0] + cr1 * inv[s][0][1];
    double c1 = cr0 * inv[s][1][0] + cr1 * inv[s][1][1];
    while (c0 >= 1) c0 += -1;
    while (c0 < 0) c0 += 1;
    while (c1 >= 1) c1 += -1;
    while (c1 < 0) c1 += 1;
    out[2 * k] = c0;
    out[2 * k + 1] = c1;
  }
  return 0;
}

int64_t oracle_targets(const oracle_h* h, const int32_t* target_sheets, int32_t num_target_sheets,
                       int64_t* out, int64_t cap) {
  int64_t c = 0;
  for (int t = 0; t < num_target_sheets; ++t) {
    int s = target_sheets[t];
    const SheetGeo& sh = h->sheets[s];
    int x_off = (sh.max0 - sh.min0) / 2, y_off = (sh.max1 - sh.min1) / 2;
    int li = sh.grid_to_index(x_off, y_off, 0);
    int64_t center = li == -1 ? -1 : li + h->sheet_base[s];
    for (int orb = 0; orb < sh.n_orb; ++orb) {
      if (c < cap) out[c] = center + orb;
      ++c;
    }
  }
  return c;
}

}  // extern "C"

// ---------------------------------------------------------------- simple-model flakes at scale

// The compact Hamiltonian of a flake of the simple model (the timed workloads)
// without the pair lists oracle_build keeps, so that flakes of 1e7 orbitals fit
// host memory: rows in the reference order (Sheet::setIndex per sheet, sheets
// in order), for each row its nearest-neighbour intralayer entries (the
// Sheet::getIntraPairs window, t = -2.7 eV on the first shell), the diagonal,
// and the interlayer entries of the sheets below and above (the
// Hstruct::getInterPairs window, in-plane distance < 12.5 A, kept where the
// 3-D distance is < 8 A), each divided by `rescale` with `shift` on the
// diagonal as generateRealH does (locality.cpp:4166-4176). Rows are built on
// `threads` host threads. Entries whose value is zero (the diagonal excepted)
// are not stored, as the device's compact copy. Returns the entry count; the
// arrays are written when cap >= that count (rowptr: n + 1 entries always).
extern "C" int64_t oracle_flake_sites(const leo2d_geom* g) {
  if (!g || !g->prepared || g->boundary_condition != 0) return -1;
  int64_t n = 0;
  for (int s = 0; s < g->num_sheets; ++s) {
    SheetGeo sh;
    make_sheet(g, s, sh);
    n += sh.max_index;
  }
  return n;
}

extern "C" int64_t oracle_simple_flake_csr(const leo2d_geom* g, double rescale, double shift, int threads,
                                           int64_t* rowptr, int32_t* col, double* val, int64_t cap) {
  if (!g || !g->prepared || g->boundary_condition != 0 || g->model != LEO2D_MODEL_SIMPLE) return -1;
  const int S = g->num_sheets;
  std::vector<SheetGeo> sheets(S);
  std::vector<int64_t> base(S + 1, 0);
  for (int s = 0; s < S; ++s) {
    make_sheet(g, s, sheets[s]);
    base[s + 1] = base[s] + sheets[s].max_index;
  }
  const int64_t n = base[S];
  auto pos_of = [&](int s, int i, int j, int l, double p[3]) {
    const SheetGeo& sh = sheets[s];
    double lp[3];
    sh.pos_grid(i, j, l, lp);
    const double th = g->angles[s];
    p[0] = lp[0] * std::cos(th) - lp[1] * std::sin(th);
    p[1] = lp[0] * std::sin(th) + lp[1] * std::cos(th);
    p[2] = lp[2] + g->heights[s];
  };
  // row r: visits (column, value) of its stored entries
  auto row = [&](int64_t r, auto&& emit) {
    int s = 0;
    while (r >= base[s + 1]) ++s;
    const SheetGeo& sh = sheets[s];
    const int k = (int)(r - base[s]);
    const int ih = sh.idx[3 * (size_t)k], jh = sh.idx[3 * (size_t)k + 1], l0 = sh.idx[3 * (size_t)k + 2];
    double ph[3];
    pos_of(s, ih, jh, l0, ph);
    emit((int32_t)r, shift / rescale);  // the diagonal
    double lp[3];
    sh.pos_grid(ih, jh, l0, lp);
    const int i0 = sh.find_nearest(lp, 0), j0 = sh.find_nearest(lp, 1);
    for (int i = i0 - 4; i < i0 + 4; ++i)
      for (int j = j0 - 4; j < j0 + 4; ++j)
        for (int l = 0; l < sh.n_orb; ++l) {
          const int k2 = sh.grid_to_index(i, j, l);
          if (k2 < 0 || k2 == k) continue;
          const double t = intralayer(LEO2D_MODEL_SIMPLE, l0, l, i - ih, j - jh);
          if (t != 0) emit((int32_t)(base[s] + k2), t / rescale);
        }
    for (int side = 0; side < 2; ++side) {
      const int s0 = side == 0 ? s - 1 : s + 1;
      if (s0 < 0 || s0 >= S) continue;
      const SheetGeo& o = sheets[s0];
      const double th = -g->angles[s0];
      const double xr = ph[0] * std::cos(th) - ph[1] * std::sin(th);
      const double yr = ph[0] * std::sin(th) + ph[1] * std::cos(th);
      const int ic = std::min(std::max(int(std::floor(o.a_inv[0][0] * xr + o.a_inv[0][1] * yr)), o.min0), o.max0) - o.min0;
      const int jc = std::min(std::max(int(std::floor(o.a_inv[1][0] * xr + o.a_inv[1][1] * yr)), o.min1), o.max1) - o.min1;
      for (int i = std::max(0, ic - 6); i < std::min(o.H, ic + 6); ++i)
        for (int j = std::max(0, jc - 6); j < std::min(o.W, jc + 6); ++j)
          for (int l = 0; l < o.n_orb; ++l) {
            const int k2 = o.grid_to_index(i, j, l);
            if (k2 < 0) continue;
            double p2[3];
            pos_of(s0, i, j, l, p2);
            const double dx = p2[0] - ph[0], dy = p2[1] - ph[1];
            if (dx * dx + dy * dy >= 12.5 * 12.5) continue;
            const double t = simple_inter_t(dx, dy, p2[2] - ph[2], rescale);
            if (t != 0) emit((int32_t)(base[s0] + k2), t);
          }
    }
  };
  if (threads < 1) threads = 1;
  auto parallel = [&](auto&& body) {
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
      th.emplace_back([&, t] {
        for (int64_t r = n * t / threads; r < n * (t + 1) / threads; ++r) body(r);
      });
    for (auto& x : th) x.join();
  };
  parallel([&](int64_t r) {
    int64_t c = 0;
    row(r, [&](int32_t, double) { ++c; });
    rowptr[r + 1] = c;
  });
  rowptr[0] = 0;
  for (int64_t r = 0; r < n; ++r) rowptr[r + 1] += rowptr[r];
  const int64_t nnz = rowptr[n];
  if (cap < nnz) return nnz;
  parallel([&](int64_t r) {
    int64_t e = rowptr[r];
    row(r, [&](int32_t c, double v) {
      col[e] = c;
      val[e] = v;
      ++e;
    });
  });
  return nnz;
}

// ---------------------------------------------------------------- recursions

namespace {

// SpMatrix::vectorMultiply, in-tree loop (spmatrix.cpp:346-360):
// out = alpha * H in + beta * out
void spmv(int64_t n, const int64_t* rp, const int32_t* col, const double* val, const double* in,
          double* out, double alpha, double beta) {
  for (int64_t r = 0; r < n; ++r) {
    double temp_sum = 0;
    for (int64_t i = rp[r]; i < rp[r + 1]; ++i) temp_sum += in[col[i]] * val[i];
    out[r] = alpha * temp_sum + beta * out[r];
  }
}

}  // namespace

extern "C" {

void oracle_kpm_trace(int64_t n, const int64_t* rp, const int32_t* col, const double* val,
                      int32_t R, const double* vectors, int32_t P, double* mu_out) {
  std::vector<double> Tp(n), Tj(n), Tn(n);
  for (int t = 0; t < R; ++t) {
    const double* v = vectors + (size_t)t * n;
    double* mu = mu_out + (size_t)t * P;
    for (int64_t i = 0; i < n; ++i) Tp[i] = v[i];
    std::fill(Tj.begin(), Tj.end(), 0.0);
    spmv(n, rp, col, val, Tp.data(), Tj.data(), 1, 0);
    std::fill(Tn.begin(), Tn.end(), 0.0);
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += v[i] * v[i];
    mu[0] = s;
    s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += Tj[i] * v[i];
    mu[1] = s;
    spmv(n, rp, col, val, Tj.data(), Tn.data(), 2, 0);
    for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
    for (int j = 2; j < P / 2; ++j) {
      for (int64_t c = 0; c < n; ++c) { Tp[c] = Tj[c]; Tj[c] = Tn[c]; }
      s = 0.0;
      for (int64_t i = 0; i < n; ++i) s += Tj[i] * v[i];
      mu[j] = s;
      spmv(n, rp, col, val, Tj.data(), Tn.data(), 2, 0);
      for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
      if (j >= P / 4) {
        double an_an = 0, anp_an = 0;
        for (int64_t c = 0; c < n; ++c) {
          an_an += Tj[c] * Tj[c];
          anp_an += Tn[c] * Tj[c];
        }
        mu[2 * j] = 2 * an_an - mu[0];
        mu[2 * j + 1] = 2 * anp_an - mu[1];
      }
    }
  }
}

// ---------------------------------------------------------------- complex H (magnetic field)

int64_t oracle_vacancy_reduction(int64_t n, const int64_t* orbitals, int64_t count, int64_t* reduction) {
  // workerChebSolve's loop: orbital i is removed when it equals any list entry
  std::vector<char> gone((size_t)n, 0);
  for (int64_t j = 0; j < count; ++j)
    if (orbitals[j] >= 0 && orbitals[j] < n) gone[(size_t)orbitals[j]] = 1;
  int64_t counter = 0;
  for (int64_t i = 0; i < n; ++i) {
    reduction[i] = counter;
    counter += gone[(size_t)i];
  }
  reduction[n] = counter;
  return n - counter;
}

int64_t oracle_remove_orbitals(int64_t n, const int64_t* rp, const int32_t* col, const double* v0,
                               const double* v1, const double* v2, const int64_t* red, int64_t* rp_out,
                               int32_t* col_out, double* v0_out, double* v1_out, double* v2_out) {
  // orbital i is a vacancy when reduction steps up across it
  auto removed = [&](int64_t i) { return red[i] + 1 == red[i + 1]; };
  int64_t out = 0;
  for (int64_t r = 0; r < n; ++r) {
    if (removed(r)) continue;
    rp_out[r - red[r]] = out;
    for (int64_t e = rp[r]; e < rp[r + 1]; ++e) {
      const int64_t c = col[e];
      if (removed(c)) continue;
      col_out[out] = (int32_t)(c - red[c]);
      if (v0) v0_out[out] = v0[e];
      if (v1) v1_out[out] = v1[e];
      if (v2) v2_out[out] = v2[e];
      ++out;
    }
  }
  rp_out[n - red[n]] = out;
  return out;
}

void oracle_peierls(int64_t n, const int64_t* rp, const int32_t* col, const double* val, const double* pos,
                    double B, double* re, double* im) {
  for (int64_t r = 0; r < n; ++r) {
    const double x1 = pos[3 * r], y1 = pos[3 * r + 1];
    for (int64_t e = rp[r]; e < rp[r + 1]; ++e) {
      const int64_t c = col[e];
      const double x2 = pos[3 * c], y2 = pos[3 * c + 1];
      // Locality::peierlsPhase (locality.cpp:7157-7161), then std::polar(t, phase)
      const double pre = 3.14e-5;
      const double phase = pre * B * (x2 - x1) * (0.5) * (y1 + y2);
      const std::complex<double> z = std::polar(val[e], phase);
      // v_c starts at 0 and zero couplings are skipped (locality.cpp:4928-4941)
      const std::complex<double> v = z != std::complex<double>(0.0) ? std::complex<double>(0.0) + z
                                                                    : std::complex<double>(0.0);
      re[e] = v.real();
      im[e] = v.imag();
    }
  }
}

namespace {
using cplx = std::complex<double>;
// SpMatrix::vectorMultiply, complex loop form (spmatrix.cpp:397-409)
void zspmv(int64_t n, const int64_t* rp, const int32_t* col, const cplx* v, const cplx* in, cplx* out,
           cplx alpha, cplx beta) {
  for (int64_t r = 0; r < n; ++r) {
    cplx s(0, 0);
    for (int64_t i = rp[r]; i < rp[r + 1]; ++i) s += in[col[i]] * v[i];
    out[r] = alpha * s + beta * out[r];
  }
}
std::vector<cplx> zvals(int64_t nnz, const double* re, const double* im) {
  std::vector<cplx> v((size_t)nnz);
  for (int64_t e = 0; e < nnz; ++e) v[e] = cplx(re[e], im[e]);
  return v;
}
}  // namespace

void oracle_kpm_trace_cpx(int64_t n, const int64_t* rp, const int32_t* col, const double* re,
                          const double* im, int32_t R, const double* vectors, int32_t P, double* mu_out) {
  const std::vector<cplx> V = zvals(rp[n], re, im);
  std::vector<cplx> Tp(n), Tj(n), Tn(n);
  for (int t = 0; t < R; ++t) {
    const double* v = vectors + (size_t)t * n;
    double* mu = mu_out + (size_t)t * P;
    for (int64_t i = 0; i < n; ++i) Tp[i] = v[i];
    std::fill(Tj.begin(), Tj.end(), cplx(0.0));
    zspmv(n, rp, col, V.data(), Tp.data(), Tj.data(), 1, 0);
    std::fill(Tn.begin(), Tn.end(), cplx(0.0));
    cplx s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += v[i] * v[i];
    mu[0] = s.real();
    s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += Tj[i] * v[i];
    mu[1] = s.real();
    zspmv(n, rp, col, V.data(), Tj.data(), Tn.data(), 2, 0);
    for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
    for (int j = 2; j < P / 2; ++j) {
      for (int64_t c = 0; c < n; ++c) { Tp[c] = Tj[c]; Tj[c] = Tn[c]; }
      s = 0.0;
      for (int64_t i = 0; i < n; ++i) s += Tj[i] * v[i];
      mu[j] = s.real();
      zspmv(n, rp, col, V.data(), Tj.data(), Tn.data(), 2, 0);
      for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
      if (j >= P / 4) {
        double an_an = 0, anp_an = 0;
        for (int64_t c = 0; c < n; ++c) {
          an_an += (std::conj(Tj[c]) * Tj[c]).real();
          anp_an += (std::conj(Tn[c]) * Tj[c]).real();
        }
        mu[2 * j] = 2 * an_an - mu[0];
        mu[2 * j + 1] = 2 * anp_an - mu[1];
      }
    }
  }
}

void oracle_kpm_ldos_cpx(int64_t n, const int64_t* rp, const int32_t* col, const double* re,
                         const double* im, const int64_t* targets, int64_t T, int32_t P, double* mu_out) {
  const std::vector<cplx> V = zvals(rp[n], re, im);
  std::vector<cplx> Tp(n), Tj(n), Tn(n);
  for (int64_t t = 0; t < T; ++t) {
    const int64_t ti = targets[t];
    double* mu = mu_out + (size_t)t * P;
    std::fill(Tp.begin(), Tp.end(), cplx(0.0));
    Tp[ti] = 1.0;
    std::fill(Tj.begin(), Tj.end(), cplx(0.0));
    zspmv(n, rp, col, V.data(), Tp.data(), Tj.data(), 1, 0);
    std::fill(Tn.begin(), Tn.end(), cplx(0.0));
    mu[0] = 1;
    mu[1] = Tj[ti].real();
    zspmv(n, rp, col, V.data(), Tj.data(), Tn.data(), 2, 0);
    for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
    for (int j = 2; j < P / 2; ++j) {
      for (int64_t c = 0; c < n; ++c) { Tp[c] = Tj[c]; Tj[c] = Tn[c]; }
      mu[j] = Tj[ti].real();
      zspmv(n, rp, col, V.data(), Tj.data(), Tn.data(), 2, 0);
      for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
      if (j >= P / 4) {
        double an_an = 0, anp_an = 0;
        for (int64_t c = 0; c < n; ++c) {
          an_an += (std::conj(Tj[c]) * Tj[c]).real();
          anp_an += (std::conj(Tn[c]) * Tj[c]).real();
        }
        mu[2 * j] = 2 * an_an - mu[0];
        mu[2 * j + 1] = 2 * anp_an - mu[1];
      }
    }
  }
}

void oracle_kpm_trace_cpx_doubling(int64_t n, const int64_t* rp, const int32_t* col, const double* re,
                                   const double* im, int32_t R, const double* vre, const double* vim,
                                   int32_t P, double* mu_out) {
  const std::vector<cplx> V = zvals(rp[n], re, im);
  std::vector<cplx> Tp(n), Tj(n), Tn(n);
  for (int t = 0; t < R; ++t) {
    double* mu = mu_out + (size_t)t * P;
    for (int64_t i = 0; i < n; ++i) Tj[i] = cplx(vre[(size_t)t * n + i], vim[(size_t)t * n + i]);  // T_0
    std::fill(Tn.begin(), Tn.end(), cplx(0.0));
    zspmv(n, rp, col, V.data(), Tj.data(), Tn.data(), 1, 0);  // T_1
    double mu0 = 0, mu1 = 0;
    for (int64_t c = 0; c < n; ++c) {
      mu0 += (std::conj(Tj[c]) * Tj[c]).real();
      mu1 += (std::conj(Tn[c]) * Tj[c]).real();
    }
    mu[0] = mu0;
    mu[1] = mu1;
    for (int k = 1; k < P / 2; ++k) {
      for (int64_t c = 0; c < n; ++c) { Tp[c] = Tj[c]; Tj[c] = Tn[c]; }
      zspmv(n, rp, col, V.data(), Tj.data(), Tn.data(), 2, 0);
      for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
      double an_an = 0, anp_an = 0;
      for (int64_t c = 0; c < n; ++c) {
        an_an += (std::conj(Tj[c]) * Tj[c]).real();
        anp_an += (std::conj(Tn[c]) * Tj[c]).real();
      }
      mu[2 * k] = 2 * an_an - mu0;
      mu[2 * k + 1] = 2 * anp_an - mu1;
    }
  }
}

void oracle_kpm_trace_doubling(int64_t n, const int64_t* rp, const int32_t* col,
                               const double* val, int32_t R, const double* vectors, int32_t P,
                               double* mu_out) {
  std::vector<double> Tp(n), Tj(n), Tn(n);
  for (int t = 0; t < R; ++t) {
    const double* v = vectors + (size_t)t * n;
    double* mu = mu_out + (size_t)t * P;
    for (int64_t i = 0; i < n; ++i) Tj[i] = v[i];  // T_0
    std::fill(Tp.begin(), Tp.end(), 0.0);
    for (int k = 0; k < P / 2; ++k) {
      // T_{k+1} = 2 H T_k - T_{k-1}  (T_1 = H T_0)
      spmv(n, rp, col, val, Tj.data(), Tn.data(), k == 0 ? 1.0 : 2.0, 0);
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

void oracle_kpm_ldos(int64_t n, const int64_t* rp, const int32_t* col, const double* val,
                     const int64_t* targets, int64_t T, int32_t P, double* mu_out) {
  std::vector<double> Tp(n), Tj(n), Tn(n);
  for (int64_t t = 0; t < T; ++t) {
    const int64_t ti = targets[t];
    double* mu = mu_out + (size_t)t * P;
    std::fill(Tp.begin(), Tp.end(), 0.0);
    Tp[ti] = 1.0;
    std::fill(Tj.begin(), Tj.end(), 0.0);
    spmv(n, rp, col, val, Tp.data(), Tj.data(), 1, 0);
    std::fill(Tn.begin(), Tn.end(), 0.0);
    mu[0] = 1;
    mu[1] = Tj[ti];
    spmv(n, rp, col, val, Tj.data(), Tn.data(), 2, 0);
    for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
    for (int j = 2; j < P / 2; ++j) {
      for (int64_t c = 0; c < n; ++c) { Tp[c] = Tj[c]; Tj[c] = Tn[c]; }
      mu[j] = Tj[ti];
      spmv(n, rp, col, val, Tj.data(), Tn.data(), 2, 0);
      for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
      if (j >= P / 4) {
        double an_an = 0, anp_an = 0;
        for (int64_t c = 0; c < n; ++c) {
          an_an += Tj[c] * Tj[c];
          anp_an += Tn[c] * Tj[c];
        }
        mu[2 * j] = 2 * an_an - mu[0];
        mu[2 * j + 1] = 2 * anp_an - mu[1];
      }
    }
  }
}

void oracle_kpm_cond(int64_t n, const int64_t* rp, const int32_t* col, const double* val,
                     const double* val_dx, const int64_t* targets, int64_t T, int32_t P,
                     double* out) {
  std::vector<double> beta((size_t)n * P), Tp(n), Tj(n), Tn(n), a0(n), tmp(n), e(n);
  for (int64_t t = 0; t < T; ++t) {
    const int64_t ti = targets[t];
    // alpha_0 = -dxH e_t (locality.cpp:4326-4359)
    std::fill(e.begin(), e.end(), 0.0);
    e[ti] = 1;
    std::fill(tmp.begin(), tmp.end(), 0.0);
    spmv(n, rp, col, val_dx, e.data(), tmp.data(), 1, 0);
    for (int64_t i = 0; i < n; ++i) a0[i] = -tmp[i];
    // beta_m = T_m(H) e_t for m < P-1 (6471-6621)
    std::fill(beta.begin(), beta.end(), 0.0);
    std::fill(Tp.begin(), Tp.end(), 0.0);
    Tp[ti] = 1.0;
    std::fill(Tj.begin(), Tj.end(), 0.0);
    std::fill(Tn.begin(), Tn.end(), 0.0);
    for (int64_t i = 0; i < n; ++i) beta[i] = Tp[i];
    spmv(n, rp, col, val, Tp.data(), Tj.data(), 1, 0);
    for (int64_t i = 0; i < n; ++i) beta[n + i] = Tj[i];
    for (int j = 2; j < P - 1; ++j) {
      spmv(n, rp, col, val, Tj.data(), Tn.data(), 2, 0);
      for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
      for (int64_t i = 0; i < n; ++i) beta[(size_t)j * n + i] = Tn[i];
      for (int64_t c = 0; c < n; ++c) { Tp[c] = Tj[c]; Tj[c] = Tn[c]; }
    }
    // alpha side (6624-6715)
    double* C = out + (size_t)t * P * P;
    auto row = [&](const double* a, int r) {
      std::fill(tmp.begin(), tmp.end(), 0.0);
      spmv(n, rp, col, val_dx, a, tmp.data(), 1, 0);
      for (int p1 = 0; p1 < P; ++p1) {
        double s = 0;
        for (int64_t i = 0; i < n; ++i) s = s + tmp[i] * beta[(size_t)p1 * n + i];
        C[(size_t)r * P + p1] = s;
      }
    };
    for (int64_t i = 0; i < n; ++i) Tp[i] = a0[i];
    row(Tp.data(), 0);
    std::fill(Tj.begin(), Tj.end(), 0.0);
    spmv(n, rp, col, val, Tp.data(), Tj.data(), 1, 0);
    row(Tj.data(), 1);
    std::fill(Tn.begin(), Tn.end(), 0.0);
    spmv(n, rp, col, val, Tj.data(), Tn.data(), 2, 0);
    for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
    for (int j = 2; j < P; ++j) {
      for (int64_t c = 0; c < n; ++c) { Tp[c] = Tj[c]; Tj[c] = Tn[c]; }
      row(Tj.data(), j);
      spmv(n, rp, col, val, Tj.data(), Tn.data(), 2, 0);
      for (int64_t c = 0; c < n; ++c) Tn[c] = Tn[c] - Tp[c];
    }
  }
}

void oracle_kpm_cond_trace(int64_t n, const int64_t* rp, const int32_t* col,
                           const double* val, const double* val_dx, int32_t R,
                           const double* vectors, int32_t M, double* out) {
  std::vector<double> A((size_t)M * n), B((size_t)M * n), Tp(n), Tj(n), Tn(n), Dr(n);
  std::fill(out, out + (size_t)M * M, 0.0);
  auto cheb = [&](const double* start, double* dst, bool apply_d) {
    for (int64_t i = 0; i < n; ++i) Tj[i] = start[i];
    std::fill(Tp.begin(), Tp.end(), 0.0);
    for (int m = 0; m < M; ++m) {
      if (apply_d) {
        std::fill(dst + (size_t)m * n, dst + (size_t)(m + 1) * n, 0.0);
        spmv(n, rp, col, val_dx, Tj.data(), dst + (size_t)m * n, 1, 0);
      } else {
        std::copy(Tj.begin(), Tj.end(), dst + (size_t)m * n);
      }
      spmv(n, rp, col, val, Tj.data(), Tn.data(), m == 0 ? 1.0 : 2.0, 0);
      if (m > 0)
        for (int64_t c = 0; c < n; ++c) Tn[c] -= Tp[c];
      Tp.swap(Tj);
      Tj.swap(Tn);
    }
  };
  for (int v = 0; v < R; ++v) {
    const double* r = vectors + (size_t)v * n;
    std::fill(Dr.begin(), Dr.end(), 0.0);
    spmv(n, rp, col, val_dx, r, Dr.data(), 1, 0);
    cheb(Dr.data(), A.data(), false);  // a_m = T_m (D r)
    cheb(r, B.data(), true);           // b_m = D T_m r
    for (int a = 0; a < M; ++a)
      for (int b = 0; b < M; ++b) {
        double s = 0;
        const double* x = A.data() + (size_t)a * n;
        const double* y = B.data() + (size_t)b * n;
        for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
        out[(size_t)a * M + b] += s;
      }
  }
}

// Jackson coefficients as param_tools.cpp:673-676
static double jackson(int P, int i) {
  return ((P - i) * std::cos((M_PI * i) / P) + std::sin((M_PI * i) / P) / std::tan(M_PI / P)) / (P);
}

void oracle_dos_transform(const double* mu, int32_t P, int32_t num_sets, double rescale,
                          double shift, double scale, double* dos_out, double* energies_out) {
  std::vector<double> m(P, 0.0), in(P);
  if (num_sets == 1) {
    for (int i = 0; i < P; ++i) m[i] = mu[i];
  } else {
    for (int i = 0; i < P; ++i)
      for (int s = 0; s < num_sets; ++s) m[i] = m[i] + mu[(size_t)s * P + i] / ((double)num_sets);
  }
  for (int i = 0; i < P; ++i) in[i] = jackson(P, i) * m[i];
  for (int k = 0; k < P; ++k) {
    long double acc = in[0];
    for (int j = 1; j < P; ++j)
      acc += 2.0L * in[j] * std::cos((long double)M_PI * j * (k + 0.5L) / P);
    double E = shift + rescale * std::cos((k * 1.0 + 0.5) * M_PI / P);
    if (energies_out) energies_out[k] = E;
    dos_out[k] = scale * (double)acc /
                 (M_PI * std::sqrt(rescale * rescale - (E - shift) * (E - shift)));
  }
}

void oracle_dos_reconstruct(const double* mu, int32_t P, const double* E, int64_t nE,
                            double rescale, double center, double scale, double* out) {
  std::vector<double> g(P);
  for (int i = 0; i < P; ++i) g[i] = jackson(P, i) * mu[i];
  for (int64_t e = 0; e < nE; ++e) {
    double x = (E[e] - center) / rescale;
    if (!(x > -1.0 && x < 1.0)) { out[e] = 0.0; continue; }
    // Clenshaw would also do; the explicit recurrence keeps the oracle plain.
    long double t0 = 1, t1 = x, acc = g[0];
    if (P > 1) acc += 2.0L * g[1] * t1;
    for (int n = 2; n < P; ++n) {
      long double t2 = 2.0L * x * t1 - t0;
      acc += 2.0L * g[n] * t2;
      t0 = t1;
      t1 = t2;
    }
    out[e] = scale * (double)acc / (M_PI * rescale * std::sqrt(1.0 - x * x));
  }
}

void oracle_cond_transform(const double* Min, int32_t P, double* out) {
  std::vector<double> g(P), in((size_t)P * P), tmp((size_t)P * P);
  for (int i = 0; i < P; ++i)
    g[i] = ((P - i) * std::cos((M_PI * i) / P) + std::sin((M_PI * i) / P) / std::tan(M_PI / P)) /
           (std::sqrt(2.0) * P);
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j) in[(size_t)i * P + j] = 2 * g[i] * g[j] * Min[(size_t)i * P + j];
  auto c = [&](int j, int k) {
    return j == 0 ? 1.0L : 2.0L * std::cos((long double)M_PI * j * (k + 0.5L) / P);
  };
  for (int i = 0; i < P; ++i)
    for (int k = 0; k < P; ++k) {
      long double a = 0;
      for (int j = 0; j < P; ++j) a += in[(size_t)i * P + j] * c(j, k);
      tmp[(size_t)i * P + k] = (double)a;
    }
  for (int k0 = 0; k0 < P; ++k0)
    for (int k1 = 0; k1 < P; ++k1) {
      long double a = 0;
      for (int i = 0; i < P; ++i) a += tmp[(size_t)i * P + k1] * c(i, k0);
      out[(size_t)k0 * P + k1] = (double)a;
    }
}

void oracle_cond_sigma(const double* mu, int32_t M, const double* E, int64_t nE, double rescale,
                       double center, double scale, double* out) {
  std::vector<double> g(M);
  for (int i = 0; i < M; ++i) g[i] = jackson(M, i) * (i == 0 ? 1.0 : 2.0);
  std::vector<long double> T(M);
  for (int64_t e = 0; e < nE; ++e) {
    double x = (E[e] - center) / rescale;
    if (!(x > -1.0 && x < 1.0)) { out[e] = 0.0; continue; }
    T[0] = 1;
    if (M > 1) T[1] = x;
    for (int n = 2; n < M; ++n) T[n] = 2.0L * x * T[n - 1] - T[n - 2];
    long double acc = 0;
    for (int a = 0; a < M; ++a) {
      long double ra = 0;
      for (int b = 0; b < M; ++b) ra += (long double)mu[(size_t)a * M + b] * g[b] * T[b];
      acc += ra * g[a] * T[a];
    }
    out[e] = scale * (double)acc / (M_PI * M_PI * (1.0 - x * x));
  }
}

void oracle_gershgorin(int64_t n, const int64_t* rp, const int32_t* col, const double* val,
                       double* emin, double* emax) {
  double lo = INFINITY, hi = -INFINITY;
  for (int64_t r = 0; r < n; ++r) {
    double c = 0, rad = 0;
    for (int64_t i = rp[r]; i < rp[r + 1]; ++i) {
      if (col[i] == r) c += val[i];
      else rad += std::fabs(val[i]);
    }
    lo = std::min(lo, c - rad);
    hi = std::max(hi, c + rad);
  }
  *emin = lo;
  *emax = hi;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter (row_lo, row_hi,
// vec_lo, vec_hi), key (seed_lo, seed_hi). The GPU generator evaluates the same
// integer rounds.
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

void oracle_phase_vectors(uint64_t seed, uint64_t first_vector, int32_t R, int64_t n, double* re,
                          double* im) {
  for (int v = 0; v < R; ++v)
    for (int64_t i = 0; i < n; ++i) {
      uint64_t vv = first_vector + (uint64_t)v;
      uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)vv,
                       (uint32_t)(vv >> 32)};
      philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
      double u = (double)(c[0] >> 8) * (1.0 / 16777216.0);
      double phi = 6.283185307179586 * u;
      re[(size_t)v * n + i] = (double)(float)std::cos(phi);
      im[(size_t)v * n + i] = (double)(float)std::sin(phi);
    }
}

void oracle_reference_gaussian(int32_t R, int64_t n, double* out) {
  std::default_random_engine generator;
  std::normal_distribution<double> distribution(0.0, 1.0);
  for (int s = 0; s < R; ++s)
    for (int64_t i = 0; i < n; ++i) out[(size_t)s * n + i] = distribution(generator);
}

}  // extern "C"
