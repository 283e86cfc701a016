// geom.cu - GPU assembly of the tight-binding Hamiltonian.
//
// Replaces, for one job with zero sheet shifts:
//   Sheet::setIndex / posAtomGrid / checkShape   src/geom/sheet.cpp:217-285, 482-559
//   Hstruct::setIndex / posAtomIndex / findNearest src/geom/hstruct.cpp:69-288
//   Hstruct::getInterPairs (+ orderPairs)         src/geom/hstruct.cpp:298-666
//   Sheet::getIntraPairs (+ orderPairs)           src/geom/sheet.cpp:624-849
//   Locality::setConfigPositions (real space)     src/locality.cpp:3618-3642
//   Locality::generateRealH                       src/locality.cpp:3900-4321
// The CSR row pointers and column indices equal the reference's; values agree
// to within rounding of the FP64 transcendental functions.
//
// This file is compiled with -fmad=false: the reference's x86-64 build never
// fuses a multiply into an add, and site membership, search windows and the
// 12.5 A pair cutoff depend on those roundings. Products of integers and
// lattice constants, window arithmetic and squared distances are therefore
// evaluated here in the same order and rounding as the reference.
//
// Work layout
//   sites: one thread per grid cell (mask), device scan, one thread per site.
//   flake rows (no periodic images, no duplicate pairs): one warp per row;
//     candidates of the reference's search windows are evaluated 32 at a time
//     and compacted with a ballot, so the row comes out in the reference's
//     order without any sort. Two passes: count -> scan -> fill.
//   periodic rows: one CTA per row; candidates of every supercell image are
//     keyed (intra/inter, column, image), bitonic-sorted in shared memory -
//     equal to the reference's stable bubble sort by column, because the
//     image index is the generation order - and consecutive duplicates are
//     merged in that order, as generateRealH does.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "csr.cuh"

using namespace leo2d;

namespace {

constexpr int kMaxSheets = LEO2D_MAX_SHEETS;
constexpr int kIntraSearch = 4;    // (int) Graphene::intra_search_radius (graphene.h:94)
constexpr int kInterSearch = 6;    // (int) Graphene::inter_search_radius (graphene.h:95)
constexpr double kInterCutoff = 12.5;  // hstruct.cpp:310
constexpr int kIntraShellMax = 16;     // no intralayer hopping beyond this neighbour shell
constexpr int kRowWarps = 8;           // k_flake_rows: warps (rows in flight) per 256-thread block
constexpr int kInterSeg = 288;         // k_flake_rows: interlayer candidates per segment (a 12 x 12 x 2 window)

struct SheetDev {
  int min0, min1, max0, max1, H, W, n_orb;
  int stride[2][2];
  double max_R;
  double a[2][2], atom[2][3], a_inv[2][2];
  double sc[2][2], sc_inv[2][2];
  double cos_t, sin_t;    // cos/sin(angle)   (host libm, as the reference)
  double cos_mt, sin_mt;  // cos/sin(-angle)
  double s1a[2][2];       // rotated lattice of setConfigPositions
  double angle, height;
  double shift[2];        // the job's sheet shift (fractions of the rotated lattice vectors)
  int64_t base;           // first global index of the sheet
  const int32_t* grid;    // [H][W][n_orb] local index or -1
};

struct GeomDev {
  int S, model, bc, sc_search, keep_zeros, with_dx;
  double supercell[2][2];
  double rescale, shift;
  double simple_amp;  // 0.33 / rescale (the simple model's interlayer prefactor)
  double e_field;     // USE_E_FIELD's E: the diagonal gains z E (Locality::onSiteE)
  double b_field;  // non-zero: complex entries t e^{i phi} (Peierls phase)
  double kx, ky;   // Bloch vector: phases k.(r_col - r_row) per periodic image
  // the flake rows' quotients, taken once on the host (IEEE division, the same
  // bits as per entry): intra_q[r] = t(r) / rescale for the shells r <=
  // kIntraShellMax, diag_q = (t(0) + shift) / rescale (used without a field E)
  double intra_q[kIntraShellMax + 1];
  double diag_q;
  int diag_const;  // no field E: every diagonal entry is diag_q
  int cpx;         // complex entries (a field or a Bloch vector)
  int shifted;     // some sheet is shifted: values from the shifted positions
  SheetDev sh[kMaxSheets];
};

__device__ __forceinline__ void pos_grid(const SheetDev& s, int i, int j, int l, double p[3]) {
  const int ii = i + s.min0, jj = j + s.min1;
  p[0] = ii * s.a[0][0] + jj * s.a[1][0] + s.atom[l][0];
  p[1] = ii * s.a[0][1] + jj * s.a[1][1] + s.atom[l][1];
  p[2] = s.atom[l][2];
}

// Sheet::checkShape; pow(x, 2) is x*x exactly in glibc.
__device__ __forceinline__ bool check_shape(const SheetDev& s, int bc, const double p[3]) {
  if (bc == 1) {
    const double delta = 0.0, grid_delta = 0.000001;
    double i = (p[0] + delta) * s.sc_inv[0][0] + (p[1] + delta) * s.sc_inv[0][1];
    double j = (p[0] + delta) * s.sc_inv[1][0] + (p[1] + delta) * s.sc_inv[1][1];
    return i >= 0.0 - grid_delta && i < 1.0 - grid_delta && j >= 0.0 - grid_delta &&
           j < 1.0 - grid_delta;
  }
  return p[0] * p[0] + p[1] * p[1] < s.max_R * s.max_R;
}

__device__ __forceinline__ int grid_to_index(const SheetDev& s, int i, int j, int l) {
  if (i >= 0 && i < s.H && j >= 0 && j < s.W && l >= 0 && l < s.n_orb)
    return s.grid[((int64_t)i * s.W + j) * s.n_orb + l];
  return -1;
}

// Sheet::findNearest (sheet frame)
__device__ __forceinline__ int find_nearest_sheet(const SheetDev& s, const double p[3], int dim) {
  if (dim == 0) {
    double i_new = s.a_inv[0][0] * p[0] + s.a_inv[0][1] * p[1];
    return min(max(int(floor(i_new)), s.min0), s.max0) - s.min0;
  }
  double j_new = s.a_inv[1][0] * p[0] + s.a_inv[1][1] * p[1];
  return min(max(int(floor(j_new)), s.min1), s.max1) - s.min1;
}

// Hstruct::findNearest (global frame, rotated by -angle, zero shifts)
__device__ __forceinline__ int find_nearest_h(const SheetDev& s, const double p[3], int dim) {
  const double z0 = 0.0;
  double x_new = p[0] * s.cos_mt - p[1] * s.sin_mt + z0 * s.a[0][0] + z0 * s.a[1][0];
  double y_new = p[0] * s.sin_mt + p[1] * s.cos_mt + z0 * s.a[0][1] + z0 * s.a[1][1];
  if (dim == 0) {
    double i_new = s.a_inv[0][0] * x_new + s.a_inv[0][1] * y_new;
    return min(max(int(floor(i_new)), s.min0), s.max0) - s.min0;
  }
  double j_new = s.a_inv[1][0] * x_new + s.a_inv[1][1] * y_new;
  return min(max(int(floor(j_new)), s.min1), s.max1) - s.min1;
}

// Coupling::Intralayer::graphene (graphene.cpp:13-89) and the simple model:
// the neighbour shell r of a grid offset, and the shell's hopping.
__device__ __forceinline__ int intra_shell(int orow, int ocol, int d0, int d1) {
  int h0 = 2 * d0 + d1;
  const int h1 = -1 * d0 + d1;
  if (ocol == 0 && orow == 1) h0 -= 1;
  else if (ocol == 1 && orow == 0) h0 += 1;
  return h0 * (h0 + h1) + h1 * h1;
}
__host__ __device__ inline double intra_shell_t(int model, int r) {
  if (model == LEO2D_MODEL_SIMPLE) return r == 1 ? -2.7 : 0.0;
  switch (r) {
    case 0: return 0.3504;
    case 1: return -2.8922;
    case 3: return 0.2425;
    case 4: return -0.2656;
    case 7: return 0.0235;
    case 9: return 0.0524;
    case 12: return -0.0209;
    case 13: return -0.0148;
    case 16: return -0.0211;
    default: return 0.;
  }
}
__device__ __forceinline__ double intralayer(int model, int orow, int ocol, int d0, int d1) {
  return intra_shell_t(model, intra_shell(orow, ocol, d0, d1));
}

// Coupling::Interlayer::C_to_C (graphene.cpp:91-222). abs() at graphene.cpp:117
// binds to the int overload in the reference, hence the truncation. The
// fitted coefficients and the order of operations are the reference's.
__device__ double c_to_c(int orow, int ocol, double v0, double v1, double v2, double theta_row,
                         double theta_col) {
  const double kPi = 3.14159265358979323846, kPi_6 = 0.523598775598298873077;
  if (abs((int)v2) > 5) return 0;
  double r = sqrt(v0 * v0 + v1 * v1);
  if (r < 8.0) {
    double ac = atan2(v1, v0);
    double theta21 = ac - theta_row;
    if (orow == 1) theta21 += kPi_6; else theta21 -= kPi_6;
    double theta12 = ac - theta_col + kPi;
    if (ocol == 1) theta12 += kPi_6; else theta12 -= kPi_6;
    double rs = r / 2.4768;
    double z_eq = 3.35;
    double z_eps = (fabs(v2) - z_eq) / z_eq;
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
    double V0 = lambda_0 * exp(-xi_0 * (rs) * (rs)) * cos(kappa_0 * rs);
    double V3 = lambda_3 * rs * rs * exp(-xi_3 * (rs - x_3) * (rs - x_3));
    double V6 = lambda_6 * exp(-xi_6 * (rs - x_6) * (rs - x_6)) * sin(kappa_6 * rs);
    double t = V0 + V3 * (cos(3 * theta12) + cos(3 * theta21)) + V6 * (cos(6 * theta12) + cos(6 * theta21));
    double d = 8.0 - r;
    if (d < 1. && d > 0.) t *= exp(1. - 1. / (d * d));
    return t;
  }
  return 0.;
}

// Interlayer hopping divided by the energy rescale (generateRealH's
// raw_t / energy_rescale). The simple model, (0.33 / rescale) exp(-(r - 3.35) /
// 0.45) for the 3-D distance r < 8 A, takes both quotients as products (by the
// host's 0.33 / rescale and by the FP64 value of 1 / 0.45): FP64 division is
// the costly part of assembly on GB300's FP64 pipe. The reference model keeps
// the division, bit for bit.
__device__ __forceinline__ double interlayer_t(int model, int orow, int ocol, double v0, double v1, double v2,
                                               double th_row, double th_col, double rescale, double simple_amp) {
  if (model == LEO2D_MODEL_SIMPLE) {
    constexpr double kInvDecay = 1.0 / 0.45;
    const double r = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
    return r < 8.0 ? simple_amp * exp(-(r - 3.35) * kInvDecay) : 0.0;
  }
  const double v = c_to_c(orow, ocol, v0, v1, v2, th_row, th_col);
  return v != 0.0 ? v / rescale : 0.0;
}

__device__ __forceinline__ int sheet_of(const GeomDev& G, int64_t k) {
  int s = 0;
  for (int t = 1; t < G.S; ++t)
    if (k >= G.sh[t].base) s = t;
  return s;
}

// ---------------------------------------------------------------- sites

__global__ void k_site_mask(const __grid_constant__ GeomDev G, int s, int64_t* __restrict__ mask) {
  const SheetDev& sh = G.sh[s];
  const int64_t cells = (int64_t)sh.H * sh.W * sh.n_orb;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(c % sh.n_orb);
    const int64_t ij = c / sh.n_orb;
    const int j = (int)(ij % sh.W), i = (int)(ij / sh.W);
    double p[3];
    pos_grid(sh, i, j, l, p);
    mask[c] = check_shape(sh, G.bc, p) ? 1 : 0;
  }
}

__global__ void k_site_fill(int64_t cells, const int64_t* __restrict__ mask,
                            const int64_t* __restrict__ scan, int32_t* __restrict__ grid,
                            int32_t* __restrict__ site_cell) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells;
       c += (int64_t)gridDim.x * blockDim.x) {
    if (mask[c]) {
      grid[c] = (int32_t)scan[c];
      site_cell[scan[c]] = (int32_t)c;
    } else {
      grid[c] = -1;
    }
  }
}

// grid4 and i2pos of every orbital (Hstruct::setIndex, posAtomIndex, setConfigPositions).
__global__ void k_sites(const __grid_constant__ GeomDev G, int64_t n,
                        const int32_t* const* __restrict__ site_cells, int32_t* __restrict__ grid4,
                        double* __restrict__ pos, double* __restrict__ spos) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int s = sheet_of(G, k);
    const SheetDev& sh = G.sh[s];
    const int64_t c = site_cells[s][k - sh.base];
    const int l = (int)(c % sh.n_orb);
    const int64_t ij = c / sh.n_orb;
    const int j = (int)(ij % sh.W), i = (int)(ij / sh.W);
    grid4[4 * k + 0] = i;
    grid4[4 * k + 1] = j;
    grid4[4 * k + 2] = l;
    grid4[4 * k + 3] = s;
    double lp[3];
    pos_grid(sh, i, j, l, lp);
    const double z0 = 0.0;
    // index_to_pos (Hstruct::posAtomIndex with zero sheet shifts)
    double x = lp[0] * sh.cos_t - lp[1] * sh.sin_t + z0 * sh.a[0][0] + z0 * sh.a[1][0];
    double y = lp[0] * sh.sin_t + lp[1] * sh.cos_t + z0 * sh.a[0][1] + z0 * sh.a[1][1];
    double z = lp[2] + sh.height;
    // i2pos (setConfigPositions with zero job shifts): the positions the pairs come from
    pos[3 * k + 0] = x + z0 * sh.s1a[0][0] + z0 * sh.s1a[1][0];
    pos[3 * k + 1] = y + z0 * sh.s1a[0][1] + z0 * sh.s1a[1][1];
    pos[3 * k + 2] = z;
    // i2pos with the job's sheet shifts (locality.cpp:3640-3642): the values
    if (spos) {
      spos[3 * k + 0] = x + sh.shift[0] * sh.s1a[0][0] + sh.shift[1] * sh.s1a[1][0];
      spos[3 * k + 1] = y + sh.shift[0] * sh.s1a[0][1] + sh.shift[1] * sh.s1a[1][1];
      spos[3 * k + 2] = z;
    }
  }
}

// ---------------------------------------------------------------- flake rows

struct RowOut {
  int64_t* cnt_ent;
  int64_t* cnt_intra;
  int64_t* cnt_inter;
  const int64_t* rowptr;
  int32_t* col;
  double* val;
  double* dx;
  double* dy;
  double* val_im;  // imaginary parts (complex entries)
  int pad_cap;     // padded single pass: entries per row of the padded arrays
  int* overflow;   // padded single pass: set when a row has more entries than pad_cap
};

// Locality::peierlsPhase (locality.cpp:7157-7161): the phase of the hopping
// from (x1, y1) (the row's orbital) to (x2, y2) (the column's) in the field B.
__device__ __forceinline__ double peierls_phase(double x1, double x2, double y1, double y2, double B) {
  const double pre = 3.14e-5;
  return pre * B * (x2 - x1) * (0.5) * (y1 + y2);
}

// t != 0 on the integer pipe (GB300's FP64 unit is the assembly's bottleneck):
// false for +0.0 and -0.0 only, as the FP64 comparison
__device__ __forceinline__ bool t_nonzero(double t) {
  return ((unsigned long long)__double_as_longlong(t) << 1) != 0ull;
}

// One stored entry: real H (value t) or, in a field, std::polar(t, phi) as
// generateCpxH adds it (locality.cpp:4896-4941: zero couplings stay 0).
__device__ __forceinline__ void store_value(const GeomDev& G, const RowOut& out, int64_t e, double t, double x1,
                                            double y1, double x2, double y2) {
  if (!G.cpx) {
    out.val[e] = t_nonzero(t) ? t : 0.0;  // (0.0 + t of a non-zero t is t; -0.0 is stored as 0.0)
    return;
  }
  if (t == 0) {
    out.val[e] = 0.0;
    out.val_im[e] = 0.0;
    return;
  }
  // generateCpxH's phase: the Peierls phase plus k.(r2 - r1) (locality.cpp:4896-4900)
  double ph = peierls_phase(x1, x2, y1, y2, G.b_field);
  ph = ph + G.kx * (x2 - x1) + G.ky * (y2 - y1);
  double sn, cs;
  sincos(ph, &sn, &cs);  // one argument reduction for both
  out.val[e] = 0.0 + t * cs;
  out.val_im[e] = 0.0 + t * sn;
}

// A diagonal entry: (raw + shift) / rescale, with the on-site term z E of a
// perpendicular electric field (Locality::onSiteE, locality.cpp:7163-7166;
// generateRealH 4166-4172).
__device__ __forceinline__ double diag_value(const GeomDev& G, double raw, double z) {
  return G.e_field != 0.0 ? (raw + G.shift + z * G.e_field) / G.rescale : (raw + G.shift) / G.rescale;
}

// FP32 copy of the positions for the candidate prefilter of k_flake_rows.
__global__ void k_pos32(const double* __restrict__ pos, int64_t n, float4* __restrict__ p32) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    p32[k] = make_float4((float)pos[3 * k], (float)pos[3 * k + 1], (float)pos[3 * k + 2], 0.f);
}

// FP32 distances decide a candidate only when they clear a threshold by this
// margin (A). FP32 positions of up to 2^14 A are off by at most 1e-3 A, so an
// in-plane distance is off by at most 3e-3 A; nearer the threshold the FP64
// test decides, so the kept pairs and their values are those of FP64 alone.
constexpr float kPrefilterMargin = 0.05f;

// kMode 0: count entries per row; 1: fill at the scanned row pointers; 2: fill
// and count in one pass, row r at r * pad_cap of padded arrays (entries past
// pad_cap are counted, not stored, and raise `overflow`).
template <int kMode>
__global__ void __launch_bounds__(kRowWarps * 32, 3) k_flake_rows(const __grid_constant__ GeomDev G, int64_t n,
                                                    const int32_t* __restrict__ grid4,
                                                    const double* __restrict__ pos,
                                                    const float4* __restrict__ pos32,
                                                    const double* __restrict__ spos,
                                                    const float4* __restrict__ spos32, RowOut out) {
  constexpr bool kFill = kMode != 0, kPad = kMode == 2;
  // per warp: the interlayer segment's candidate codes, queue and hoppings
  __shared__ int32_t s_code[kRowWarps][kInterSeg];
  __shared__ int16_t s_queue[kRowWarps][kInterSeg];
  __shared__ double s_hop[kRowWarps][kInterSeg];
  const unsigned lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += warps) {
    const int ih = grid4[4 * row], jh = grid4[4 * row + 1], l0 = grid4[4 * row + 2],
              s = grid4[4 * row + 3];
    const SheetDev& sh = G.sh[s];
    // pos: the unshifted positions, which choose the pairs (the reference's pair
    // lists come from the unshifted geometry); spos: the job's shifted i2pos,
    // which give the values (setConfigPositions, locality.cpp:3618-3642)
    const double x1 = pos[3 * row] + 0.0, y1 = pos[3 * row + 1] + 0.0, z1 = pos[3 * row + 2];
    const double sx1 = spos[3 * row] + 0.0, sy1 = spos[3 * row + 1] + 0.0, sz1 = spos[3 * row + 2];
    int64_t o = kPad ? row * (int64_t)out.pad_cap : (kFill ? out.rowptr[row] : 0);
    const int64_t o_end = kPad ? o + out.pad_cap : 0;
    int64_t n_ent = 0, n_intra = 0, n_inter = 0;

    // intralayer: window [i0-4, i0+4) x [j0-4, j0+4) x orbitals, every candidate kept
    {
      double lp[3];
      pos_grid(sh, ih, jh, l0, lp);
      double ph[3] = {lp[0] + 0.0, lp[1] + 0.0, lp[2]};
      const int i0 = find_nearest_sheet(sh, ph, 0), j0 = find_nearest_sheet(sh, ph, 1);
      const int side = 2 * kIntraSearch;
      const int nc = side * side * sh.n_orb;
      for (int c0 = 0; c0 < nc; c0 += 32) {
        const int c = c0 + (int)lane;
        int64_t k2g = -1;
        double t = 0.0;
        if (c < nc) {
          const int l = c % sh.n_orb;
          const int j = j0 - kIntraSearch + (c / sh.n_orb) % side;
          const int i = i0 - kIntraSearch + c / (sh.n_orb * side);
          const int k2 = grid_to_index(sh, i, j, l);
          if (k2 != -1) {
            k2g = k2 + sh.base;
            // the quotients by the rescale from the host's table; a field E
            // makes the diagonal depend on the orbital's height
            const int r = intra_shell(l0, l, i - ih, j - jh);
            if (k2g == row)
              t = G.diag_const ? G.diag_q : diag_value(G, intra_shell_t(G.model, r), sz1);
            else
              t = r <= kIntraShellMax ? G.intra_q[r] : 0.0;
          }
        }
        const bool keep = k2g >= 0;
        // without KEEP_ZEROS the diagonal stays so a later rescale can shift it
        const bool store = keep && (G.keep_zeros || t_nonzero(t) || k2g == row);
        const unsigned m = __ballot_sync(0xffffffffu, store);
        n_intra += __popc(__ballot_sync(0xffffffffu, keep));
        if (kFill && store && (!kPad || o + __popc(m & lt_mask) < o_end)) {
          const int64_t e = o + __popc(m & lt_mask);
          out.col[e] = (int32_t)k2g;
          const double x2 = spos[3 * k2g], y2 = spos[3 * k2g + 1];
          store_value(G, out, e, t, sx1, sy1, x2, y2);
          if (G.with_dx) {
            out.dx[e] = t != 0 ? 0.0 + (sx1 - x2) * t : 0.0;
            out.dy[e] = t != 0 ? 0.0 + (sy1 - y2) * t : 0.0;
          }
        }
        o += __popc(m);
        n_ent += __popc(m);
      }
    }

    // interlayer: sheet below, then sheet above; window +-6 clipped; d_xy < 12.5 A.
    // Most candidates of the window have no hopping (beyond 8 A), so the FP64
    // hoppings are not taken where the candidates fall, which would leave most
    // lanes of GB300's small FP64 unit idle. Per segment of up to kInterSeg
    // candidates: (1) the FP32 tests mark each candidate (outside the window;
    // inside without a hopping to evaluate; inside with one) and queue the
    // last kind in the warp's shared memory, in candidate order; (2) the FP64
    // hoppings of the queue, on every lane; (3) the entries in candidate
    // order, as a single pass would write them.
    {
      const double ph[3] = {x1, y1, z1};
      const float x1f = (float)x1, y1f = (float)y1;
      const float sx1f = (float)sx1, sy1f = (float)sy1, sz1f = (float)sz1;
      constexpr float kWinLo = (float)(kInterCutoff - kPrefilterMargin), kWinHi = (float)(kInterCutoff + kPrefilterMargin);
      // every hopping is zero from 8 A on (in-plane for the reference model, 3-D for the simple one)
      constexpr float kHopHi = 8.0f + kPrefilterMargin, kHopLo = 8.0f - kPrefilterMargin;
      int32_t* const seg_code = s_code[threadIdx.x >> 5];
      int16_t* const seg_queue = s_queue[threadIdx.x >> 5];
      double* const seg_t = s_hop[threadIdx.x >> 5];
      for (int side_k = 0; side_k < 2; ++side_k) {
        const int s0 = side_k == 0 ? s - 1 : s + 1;
        if (s0 < 0 || s0 >= G.S) continue;
        const SheetDev& o0 = G.sh[s0];
        const int i0 = find_nearest_h(o0, ph, 0), j0 = find_nearest_h(o0, ph, 1);
        const int ilo = max(0, i0 - kInterSearch), ihi = min(o0.H, i0 + kInterSearch);
        const int jlo = max(0, j0 - kInterSearch), jhi = min(o0.W, j0 + kInterSearch);
        if (ihi <= ilo || jhi <= jlo) continue;
        const int wj = jhi - jlo;
        const int nc = (ihi - ilo) * wj * o0.n_orb;
        for (int seg0 = 0; seg0 < nc; seg0 += kInterSeg) {
          const int seg_n = min(kInterSeg, nc - seg0);
          // (1) code: -1 outside the window, else the column with bit 31 set
          // when its hopping is to be evaluated (columns are below 2^31 - 1)
          int qn = 0;
          for (int c0 = 0; c0 < seg_n; c0 += 32) {
            const int slot = c0 + (int)lane;
            bool queue = false;
            if (slot < seg_n) {
              const int c = seg0 + slot;
              int32_t code = -1;
              const int l = c % o0.n_orb;
              const int j = jlo + (c / o0.n_orb) % wj;
              const int i = ilo + c / (o0.n_orb * wj);
              const int k2 = grid_to_index(o0, i, j, l);
              if (k2 != -1) {
                const int64_t kk = k2 + o0.base;
                const float4 q = pos32[kk];
                const float dxf = q.x - x1f, dyf = q.y - y1f;
                const float d2f = dxf * dxf + dyf * dyf;
                bool in_window;
                if (d2f < kWinLo * kWinLo) {
                  in_window = true;
                } else if (d2f > kWinHi * kWinHi) {
                  in_window = false;
                } else {
                  const double x2 = pos[3 * kk], y2 = pos[3 * kk + 1];
                  in_window = (x2 - ph[0]) * (x2 - ph[0]) + (y2 - ph[1]) * (y2 - ph[1]) < kInterCutoff * kInterCutoff;
                }
                if (in_window) {
                  // the hopping cutoffs test the shifted positions
                  const float4 sq = G.shifted ? spos32[kk] : q;
                  const float hdx = sq.x - sx1f, hdy = sq.y - sy1f, hdz = sq.z - sz1f;
                  const float hd2 = hdx * hdx + hdy * hdy;
                  const float h2f = G.model == LEO2D_MODEL_SIMPLE ? hd2 + hdz * hdz : hd2;
                  queue = (kFill || !G.keep_zeros) && h2f < kHopHi * kHopHi;
                  code = (int32_t)((uint32_t)kk | (queue ? 0x80000000u : 0u));
                }
              }
              seg_code[slot] = code;
            }
            const unsigned qm = __ballot_sync(0xffffffffu, queue);
            if (queue) seg_queue[qn + __popc(qm & lt_mask)] = (int16_t)slot;
            qn += __popc(qm);
          }
          __syncwarp();
          // (2) the queued hoppings
          for (int q0 = 0; q0 < qn; q0 += 32) {
            const int qi = q0 + (int)lane;
            if (qi < qn) {
              const int slot = seg_queue[qi];
              const int64_t kk = (int64_t)((uint32_t)seg_code[slot] & 0x7fffffffu);
              double t;
              if (!kFill && !G.keep_zeros && G.model == LEO2D_MODEL_SIMPLE) {
                // counting only needs t != 0: the simple model's hopping (and its
                // quotient by a finite rescale) is non-zero exactly when the FP64
                // distance of `interlayer` is below 8 A; FP32 decides away from 8 A
                const float4 sq = G.shifted ? spos32[kk] : pos32[kk];
                const float hdx = sq.x - sx1f, hdy = sq.y - sy1f, hdz = sq.z - sz1f;
                bool nz = hdx * hdx + hdy * hdy + hdz * hdz < kHopLo * kHopLo;
                if (!nz) {
                  const double v0 = spos[3 * kk] - sx1, v1 = spos[3 * kk + 1] - sy1, v2 = spos[3 * kk + 2] - sz1;
                  nz = sqrt(v0 * v0 + v1 * v1 + v2 * v2) < 8.0;
                }
                t = nz ? 1.0 : 0.0;
              } else {
                const int l = (seg0 + slot) % o0.n_orb;
                const double x2 = spos[3 * kk], y2 = spos[3 * kk + 1], z2 = spos[3 * kk + 2];
                t = interlayer_t(G.model, l0, l, x2 - sx1, y2 - sy1, z2 - sz1, sh.angle, o0.angle, G.rescale,
                                 G.simple_amp);
              }
              seg_t[qi] = t;
            }
          }
          __syncwarp();
          // (3) the entries, in candidate order
          int qr = 0;
          for (int c0 = 0; c0 < seg_n; c0 += 32) {
            const int slot = c0 + (int)lane;
            int64_t k2g = -1;
            bool queued = false;
            if (slot < seg_n) {
              const int32_t code = seg_code[slot];
              if (code != -1) {
                k2g = (int64_t)((uint32_t)code & 0x7fffffffu);
                queued = code < 0;
              }
            }
            const unsigned qm = __ballot_sync(0xffffffffu, queued);
            const double t = queued ? seg_t[qr + __popc(qm & lt_mask)] : 0.0;
            qr += __popc(qm);
            const bool keep = k2g >= 0;
            const bool store = keep && (G.keep_zeros || t_nonzero(t));
            const unsigned m = __ballot_sync(0xffffffffu, store);
            n_inter += __popc(__ballot_sync(0xffffffffu, keep));
            if (kFill && store && (!kPad || o + __popc(m & lt_mask) < o_end)) {
              const int64_t e = o + __popc(m & lt_mask);
              out.col[e] = (int32_t)k2g;
              const double x2 = spos[3 * k2g], y2 = spos[3 * k2g + 1];
              store_value(G, out, e, t, sx1, sy1, x2, y2);
              if (G.with_dx) {
                out.dx[e] = t != 0 ? 0.0 + (sx1 - x2) * t : 0.0;
                out.dy[e] = t != 0 ? 0.0 + (sy1 - y2) * t : 0.0;
              }
            }
            o += __popc(m);
            n_ent += __popc(m);
          }
          __syncwarp();
        }
      }
    }
    if ((!kFill || kPad) && lane == 0) {
      out.cnt_ent[row] = n_ent;
      out.cnt_intra[row] = n_intra;
      out.cnt_inter[row] = n_inter;
      if (kPad && n_ent > out.pad_cap) atomicOr(out.overflow, 1);
    }
  }
}

// Copies each row's entries from the padded arrays of the single pass into the
// CSR arrays (a warp per row).
__global__ void k_unpad_rows(int64_t n, int cap, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ pcol,
                             const double* __restrict__ pval, const double* __restrict__ pdx,
                             const double* __restrict__ pdy, const double* __restrict__ pim, RowOut out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
    const int64_t o = rowptr[r], len = rowptr[r + 1] - o, src = r * (int64_t)cap;
    for (int64_t i = lane; i < len; i += 32) {
      out.col[o + i] = pcol[src + i];
      out.val[o + i] = pval[src + i];
      if (pdx) out.dx[o + i] = pdx[src + i];
      if (pdy) out.dy[o + i] = pdy[src + i];
      if (pim) out.val_im[o + i] = pim[src + i];
    }
  }
}

// ---------------------------------------------------------------- periodic rows

constexpr uint64_t kKeyInter = 1ull << 48;
constexpr uint64_t kKeyPad = ~0ull;

__device__ __forceinline__ void image_of(int img, int ss, int& dxs, int& dys) {
  const int side = 2 * ss + 1;
  dxs = img / side - ss;
  dys = img % side - ss;
}

// Value of one candidate (row, k2, image), generateRealH's rescaling included
// (generateCpxH, for complex entries, shifts the home image's diagonal only:
// locality.cpp:4885).
__device__ double periodic_value(const GeomDev& G, int64_t row, const int32_t* grid4,
                                 const double* pos, bool inter, int64_t k2, int img,
                                 double& x1, double& y1) {
  int dxs, dys;
  image_of(img, G.sc_search, dxs, dys);
  const int ih = grid4[4 * row], jh = grid4[4 * row + 1], l0 = grid4[4 * row + 2],
            s = grid4[4 * row + 3];
  const double shx = dxs * G.supercell[0][0] + dys * G.supercell[1][0];
  const double shy = dxs * G.supercell[0][1] + dys * G.supercell[1][1];
  x1 = pos[3 * row] + shx;
  y1 = pos[3 * row + 1] + shy;
  const int i2 = grid4[4 * k2], j2 = grid4[4 * k2 + 1], l2 = grid4[4 * k2 + 2], s2 = grid4[4 * k2 + 3];
  if (!inter) {
    const SheetDev& sh = G.sh[s];
    int gd0 = i2 - ih, gd1 = j2 - jh;
    gd0 = gd0 - dxs * sh.stride[0][0] - dys * sh.stride[1][0];
    gd1 = gd1 - dxs * sh.stride[0][1] - dys * sh.stride[1][1];
    const double raw = intralayer(G.model, l0, l2, gd0, gd1);
    const bool diag = k2 == row && (!G.cpx || (dxs == 0 && dys == 0));
    return diag ? diag_value(G, raw, pos[3 * row + 2]) : raw / G.rescale;
  }
  const double z1 = pos[3 * row + 2];
  const double x2 = pos[3 * k2], y2 = pos[3 * k2 + 1], z2 = pos[3 * k2 + 2];
  return interlayer_t(G.model, l0, l2, x2 - x1, y2 - y1, z2 - z1, G.sh[s].angle, G.sh[s2].angle, G.rescale,
                      G.simple_amp);
}

__device__ void block_bitonic_sort(uint64_t* keys, int n2) {
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const uint64_t a = keys[i], b = keys[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            keys[i] = b;
            keys[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

template <bool kFill>
__global__ void __launch_bounds__(256) k_periodic_rows(const __grid_constant__ GeomDev G, int64_t n,
                                                       const int32_t* __restrict__ grid4,
                                                       const double* __restrict__ pos,
                                                       const double* __restrict__ spos, int cap,
                                                       RowOut out, int* status) {
  extern __shared__ uint64_t keys[];
  __shared__ int cnt, n_intra_s, n_inter_s, n_run;
  __shared__ int warp_sums[8];
  const int ss = G.sc_search;
  const int n_img = (2 * ss + 1) * (2 * ss + 1);
  for (int64_t row = blockIdx.x; row < n; row += gridDim.x) {
    if (threadIdx.x == 0) { cnt = 0; n_intra_s = 0; n_inter_s = 0; }
    __syncthreads();
    const int ih = grid4[4 * row], jh = grid4[4 * row + 1], l0 = grid4[4 * row + 2],
              s = grid4[4 * row + 3];
    const SheetDev& sh = G.sh[s];
    double lp[3];
    pos_grid(sh, ih, jh, l0, lp);
    const double khx = pos[3 * row], khy = pos[3 * row + 1], khz = pos[3 * row + 2];

    // intralayer candidates of every image (Sheet::getIntraPairs)
    const int side = 2 * kIntraSearch;
    const int per_img = side * side * sh.n_orb;
    for (int c = threadIdx.x; c < n_img * per_img; c += blockDim.x) {
      const int img = c / per_img, cc = c % per_img;
      int dxs, dys;
      image_of(img, ss, dxs, dys);
      const double scx = dxs * sh.sc[0][0] + dys * sh.sc[1][0];
      const double scy = dxs * sh.sc[0][1] + dys * sh.sc[1][1];
      double ph[3] = {lp[0] + scx, lp[1] + scy, lp[2]};
      const int i0 = find_nearest_sheet(sh, ph, 0), j0 = find_nearest_sheet(sh, ph, 1);
      const int l = cc % sh.n_orb;
      const int j = j0 - kIntraSearch + (cc / sh.n_orb) % side;
      const int i = i0 - kIntraSearch + cc / (sh.n_orb * side);
      const int k2 = grid_to_index(sh, i, j, l);
      if (k2 == -1) continue;
      int gd0 = i - ih, gd1 = j - jh;
      gd0 = gd0 - dxs * sh.stride[0][0] - dys * sh.stride[1][0];
      gd1 = gd1 - dxs * sh.stride[0][1] - dys * sh.stride[1][1];
      const double raw = intralayer(G.model, l0, l, gd0, gd1);
      const bool keep = raw != 0 || (dxs == 0 && dys == 0);
      if (!keep) continue;
      atomicAdd(&n_intra_s, 1);
      const int64_t k2g = k2 + sh.base;
      if (!G.keep_zeros) {
        const double t = k2g == row ? (raw + G.shift) / G.rescale : raw / G.rescale;
        if (t == 0 && k2g != row) continue;
      }
      const int slot = atomicAdd(&cnt, 1);
      if (slot < cap) keys[slot] = ((uint64_t)k2g << 16) | (uint64_t)img;
    }
    // interlayer candidates of every image (Hstruct::getInterPairs)
    for (int img = 0; img < n_img; ++img) {
      int dxs, dys;
      image_of(img, ss, dxs, dys);
      const double scx = dxs * G.supercell[0][0] + dys * G.supercell[1][0];
      const double scy = dxs * G.supercell[0][1] + dys * G.supercell[1][1];
      const double ph[3] = {khx + scx, khy + scy, khz};
      for (int side_k = 0; side_k < 2; ++side_k) {
        const int s0 = side_k == 0 ? s - 1 : s + 1;
        if (s0 < 0 || s0 >= G.S) continue;
        const SheetDev& o0 = G.sh[s0];
        const int i0 = find_nearest_h(o0, ph, 0), j0 = find_nearest_h(o0, ph, 1);
        const int ilo = max(0, i0 - kInterSearch), ihi = min(o0.H, i0 + kInterSearch);
        const int jlo = max(0, j0 - kInterSearch), jhi = min(o0.W, j0 + kInterSearch);
        if (ihi <= ilo || jhi <= jlo) continue;
        const int wj = jhi - jlo;
        const int nc = (ihi - ilo) * wj * o0.n_orb;
        for (int c = threadIdx.x; c < nc; c += blockDim.x) {
          const int l = c % o0.n_orb;
          const int j = jlo + (c / o0.n_orb) % wj;
          const int i = ilo + c / (o0.n_orb * wj);
          const int k2 = grid_to_index(o0, i, j, l);
          if (k2 == -1) continue;
          const int64_t kk = k2 + o0.base;
          const double x2 = pos[3 * kk], y2 = pos[3 * kk + 1];
          if (!((x2 - ph[0]) * (x2 - ph[0]) + (y2 - ph[1]) * (y2 - ph[1]) <
                kInterCutoff * kInterCutoff))
            continue;
          atomicAdd(&n_inter_s, 1);
          if (!G.keep_zeros) {
            double xx, yy;
            const double t = periodic_value(G, row, grid4, spos, true, kk, img, xx, yy);
            if (t == 0) continue;
          }
          const int slot = atomicAdd(&cnt, 1);
          if (slot < cap) keys[slot] = kKeyInter | ((uint64_t)kk << 16) | (uint64_t)img;
        }
      }
    }
    __syncthreads();
    const int m = cnt;
    if (m > cap) {
      if (threadIdx.x == 0) atomicExch(status, kStatusBadIndex);
      __syncthreads();
      continue;
    }
    int n2 = 1;
    while (n2 < m) n2 <<= 1;
    for (int i = m + threadIdx.x; i < n2; i += blockDim.x) keys[i] = kKeyPad;
    __syncthreads();
    block_bitonic_sort(keys, n2);

    // one output entry per run of equal (intra/inter, column)
    if (!kFill) {
      int local = 0;
      for (int p = threadIdx.x; p < m; p += blockDim.x)
        if (p == m - 1 || (keys[p] >> 16) != (keys[p + 1] >> 16)) ++local;
      if (threadIdx.x == 0) n_run = 0;
      __syncthreads();
      atomicAdd(&n_run, local);
      __syncthreads();
      if (threadIdx.x == 0) {
        out.cnt_ent[row] = n_run;
        out.cnt_intra[row] = n_intra_s;
        out.cnt_inter[row] = n_inter_s;
      }
      __syncthreads();
      continue;
    }
    // fill: ordered slots by a block-wide scan of run-end flags, chunk by chunk
    int64_t base_out = out.rowptr[row];
    for (int p0 = 0; p0 < m; p0 += blockDim.x) {
      const int p = p0 + threadIdx.x;
      const bool end = p < m && (p == m - 1 || (keys[p] >> 16) != (keys[p + 1] >> 16));
      const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      const unsigned bal = __ballot_sync(0xffffffffu, end);
      if (lane == 0) warp_sums[warp] = __popc(bal);
      __syncthreads();
      int before = 0, total = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        if (w < (int)warp) before += warp_sums[w];
        total += warp_sums[w];
      }
      before += __popc(bal & ((1u << lane) - 1u));
      if (end) {
        int q = p;
        while (q > 0 && (keys[q - 1] >> 16) == (keys[p] >> 16)) --q;
        const bool inter = (keys[p] & kKeyInter) != 0;
        const int64_t k2 = (int64_t)((keys[p] >> 16) & 0xffffffffull);
        double v = 0.0, vdx = 0.0, vdy = 0.0, vim = 0.0;
        for (int e = q; e <= p; ++e) {
          const int img = (int)(keys[e] & 0xffffull);
          double x1, y1;
          const double t = periodic_value(G, row, grid4, spos, inter, k2, img, x1, y1);
          if (t != 0) {
            if (G.cpx) {
              // std::polar(t, phase) summed over the images, the phase the Peierls
              // phase plus k.(r2 - r1) with r1 the row's orbital shifted by the
              // image (locality.cpp:4718-4738, 4896-4941)
              const double x2 = spos[3 * k2], y2 = spos[3 * k2 + 1];
              double ph = peierls_phase(x1, x2, y1, y2, G.b_field);
              ph = ph + G.kx * (x2 - x1) + G.ky * (y2 - y1);
              double sn, cs;
              sincos(ph, &sn, &cs);
              v += t * cs;
              vim += t * sn;
            } else {
              v += t;
            }
            vdx += (x1 - spos[3 * k2]) * t;
            vdy += (y1 - spos[3 * k2 + 1]) * t;
          }
        }
        const int64_t e = base_out + before;
        out.col[e] = (int32_t)k2;
        out.val[e] = v;
        if (G.cpx) out.val_im[e] = vim;
        if (G.with_dx) {
          out.dx[e] = vdx;
          out.dy[e] = vdy;
        }
      }
      base_out += total;
      __syncthreads();
    }
  }
}

__global__ void k_pack_ent(const int32_t* __restrict__ col, const float* __restrict__ v, uint2* __restrict__ e,
                           int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    e[i] = make_uint2((unsigned)col[i], __float_as_uint(v[i]));
}

__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// ---------------------------------------------------------------- disregistry

// Inverse of each sheet's rotated unit cell (computed on the host with the
// same libm calls as the reference).
struct CellInv {
  double inv[2][2][2];
};

// Hstruct::getShiftConfigs (src/geom/hstruct.cpp:672-820), bilayers: the
// fractional offset of orbital k's cell site (orbital 0) from the site of the
// other sheet that Hstruct::findNearest picks, in the other sheet's rotated
// lattice, wrapped to [0,1) by the reference's loops.
__global__ void k_shift_configs(const __grid_constant__ GeomDev G, const CellInv ci, int64_t n,
                                const int32_t* __restrict__ grid4, double* __restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int s_here = grid4[4 * k + 3];
    const int s = s_here == 0 ? 1 : 0;
    const SheetDev& a = G.sh[s_here];
    const SheetDev& b = G.sh[s];
    double orig[3];
    pos_grid(a, grid4[4 * k], grid4[4 * k + 1], 0, orig);
    double here[3];
    here[0] = a.cos_t * orig[0] - a.sin_t * orig[1];
    here[1] = a.sin_t * orig[0] + a.cos_t * orig[1];
    here[2] = 0.0;
    const int ni = find_nearest_h(b, here, 0), nj = find_nearest_h(b, here, 1);
    double sp[3];
    pos_grid(b, ni, nj, 0, sp);
    const double np0 = b.cos_t * sp[0] - b.sin_t * sp[1];
    const double np1 = b.sin_t * sp[0] + b.cos_t * sp[1];
    const double cr0 = here[0] - np0, cr1 = here[1] - np1;
    double c0 = cr0 * ci.inv[s][0][0] + cr1 * ci.inv[s][0][1];
    double c1 = cr0 * ci.inv[s][1][0] + cr1 * ci.inv[s][1][1];
    while (c0 >= 1) c0 += -1;
    while (c0 < 0) c0 += 1;
    while (c1 >= 1) c1 += -1;
    while (c1 < 0) c1 += 1;
    out[2 * k] = c0;
    out[2 * k + 1] = c1;
  }
}

// ---------------------------------------------------------------- host

void fill_sheet(const leo2d_geom& g, int s, SheetDev& d) {
  d.min0 = g.min_shape[s][0];
  d.min1 = g.min_shape[s][1];
  d.max0 = g.max_shape[s][0];
  d.max1 = g.max_shape[s][1];
  d.H = d.max0 - d.min0;
  d.W = d.max1 - d.min1;
  d.n_orb = 2;
  d.max_R = g.max_R[s];
  d.shift[0] = g.shifts[s][0];
  d.shift[1] = g.shifts[s][1];
  const double a = g.model == LEO2D_MODEL_SIMPLE ? 2.46 : 2.4768;
  for (int x = 0; x < 2; ++x)
    for (int y = 0; y < 2; ++y) d.a[x][y] = g.lattice[s][x][y];
  // Graphene::atom_pos (graphene.h:82-85)
  d.atom[0][0] = 0.; d.atom[0][1] = 0.; d.atom[0][2] = 0.;
  d.atom[1][0] = 0.5 * a; d.atom[1][1] = 0.288675134594812882255 * a; d.atom[1][2] = 0;
  const double a11 = d.a[0][0], a12 = d.a[0][1], a21 = d.a[1][0], a22 = d.a[1][1];
  const double det_a = a11 * a22 - a12 * a21;
  d.a_inv[0][0] = a22 / det_a;
  d.a_inv[0][1] = -a21 / det_a;
  d.a_inv[1][0] = -a12 / det_a;
  d.a_inv[1][1] = a11 / det_a;
  std::memset(d.sc, 0, sizeof(d.sc));
  std::memset(d.sc_inv, 0, sizeof(d.sc_inv));
  std::memset(d.stride, 0, sizeof(d.stride));
  if (g.boundary_condition == 1) {
    for (int x = 0; x < 2; ++x)
      for (int y = 0; y < 2; ++y) {
        d.sc[x][y] = g.sheet_supercell[s][x][y];
        d.stride[x][y] = g.sheet_sc_stride[s][x][y];
      }
    const double det = d.sc[0][0] * d.sc[1][1] - d.sc[0][1] * d.sc[1][0];
    d.sc_inv[0][0] = d.sc[1][1] / det;
    d.sc_inv[0][1] = -d.sc[1][0] / det;
    d.sc_inv[1][0] = -d.sc[0][1] / det;
    d.sc_inv[1][1] = d.sc[0][0] / det;
  }
  d.angle = g.angles[s];
  d.height = g.heights[s];
  d.cos_t = std::cos(d.angle);
  d.sin_t = std::sin(d.angle);
  const double mt = -d.angle;
  d.cos_mt = std::cos(mt);
  d.sin_mt = std::sin(mt);
  for (int x = 0; x < 2; ++x) {
    d.s1a[x][0] = std::cos(d.angle) * d.a[x][0] - std::sin(d.angle) * d.a[x][1];
    d.s1a[x][1] = std::sin(d.angle) * d.a[x][0] + std::cos(d.angle) * d.a[x][1];
  }
  d.base = 0;
  d.grid = nullptr;
}

void validate_geom(const leo2d_geom* g) {
  LEO_REQUIRE(g, "geometry is NULL");
  LEO_REQUIRE(g->prepared, "geometry not prepared: call leo2d_geom_prepare first");
  LEO_REQUIRE(g->num_sheets >= 1 && g->num_sheets <= kMaxSheets, "num_sheets must be 1..8");
  LEO_REQUIRE(g->model == LEO2D_MODEL_REF || g->model == LEO2D_MODEL_SIMPLE, "unknown model");
  LEO_REQUIRE(g->boundary_condition == 0 || g->boundary_condition == 1,
              "boundary_condition must be 0 or 1");
  LEO_REQUIRE(g->energy_rescale != 0.0 && std::isfinite(g->energy_rescale),
              "energy_rescale must be finite and non-zero");
  LEO_REQUIRE(std::isfinite(g->energy_shift), "energy_shift must be finite");
  for (int s = 0; s < g->num_sheets; ++s) {
    LEO_REQUIRE(g->max_shape[s][0] > g->min_shape[s][0] && g->max_shape[s][1] > g->min_shape[s][1],
                "MAXSIZE must exceed MINSIZE");
    const int64_t cells = (int64_t)(g->max_shape[s][0] - g->min_shape[s][0]) *
                          (g->max_shape[s][1] - g->min_shape[s][1]) * 2;
    LEO_REQUIRE(cells < (1ll << 31), "grid too large");
    LEO_REQUIRE(std::isfinite(g->angles[s]) && std::isfinite(g->heights[s]),
                "angles and heights must be finite");
  }
  if (g->boundary_condition == 1)
    LEO_REQUIRE(g->sc_search_size >= 0 && g->sc_search_size <= 3, "sc_search_size must be 0..3");
  LEO_REQUIRE(std::isfinite(g->b_field), "b_field must be finite");
  LEO_REQUIRE(std::isfinite(g->k_vec[0]) && std::isfinite(g->k_vec[1]), "k_vec must be finite");
  LEO_REQUIRE(std::isfinite(g->e_field), "e_field must be finite");
  for (int s = 0; s < LEO2D_MAX_SHEETS; ++s)
    LEO_REQUIRE(std::isfinite(g->shifts[s][0]) && std::isfinite(g->shifts[s][1]) &&
                    std::fabs(g->shifts[s][0]) <= 1.0 && std::fabs(g->shifts[s][1]) <= 1.0,
                "sheet shifts must be finite fractions of the lattice vectors (|shift| <= 1)");
}

}  // namespace

namespace leo2d {
void csr_alloc_rowptr(leo2d_ctx* ctx, leo2d_csr* csr, int64_t n) {
  csr->rowptr.alloc(n + 1 + kCsrPad);
  LEO_CUDA(cudaMemsetAsync(csr->rowptr.p + n + 1, 0, kCsrPad * sizeof(int64_t), ctx->stream));
}

void csr_alloc_entries(leo2d_ctx* ctx, leo2d_csr* csr, int64_t nnz, bool with_dx) {
  csr->col.alloc(nnz + kCsrPad);
  csr->val64.alloc(nnz + kCsrPad);
  LEO_CUDA(cudaMemsetAsync(csr->col.p + nnz, 0, kCsrPad * sizeof(int32_t), ctx->stream));
  LEO_CUDA(cudaMemsetAsync(csr->val64.p + nnz, 0, kCsrPad * sizeof(double), ctx->stream));
  if (with_dx) {
    csr->dx64.alloc(nnz + kCsrPad);
    csr->dy64.alloc(nnz + kCsrPad);
    LEO_CUDA(cudaMemsetAsync(csr->dx64.p + nnz, 0, kCsrPad * sizeof(double), ctx->stream));
    LEO_CUDA(cudaMemsetAsync(csr->dy64.p + nnz, 0, kCsrPad * sizeof(double), ctx->stream));
  }
}

void csr_refresh_fp32(leo2d_ctx* ctx, leo2d_csr* csr) {
  csr->tile_rows_cached = 0;
  csr_drop_reordered(csr);
  if (csr->nnz == 0) return;
  csr->val32.alloc(csr->nnz + kCsrPad);
  LEO_CUDA(cudaMemsetAsync(csr->val32.p + csr->nnz, 0, kCsrPad * sizeof(float), ctx->stream));
  csr->ent.alloc(csr->nnz + kCsrPad);
  LEO_CUDA(cudaMemsetAsync(csr->ent.p + csr->nnz, 0, kCsrPad * sizeof(uint2), ctx->stream));
  launch(ctx, "to_f32", [&] {
    k_to_f32<<<grid_for(csr->nnz, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
        csr->val64.p, csr->val32.p, csr->nnz);
  });
  launch(ctx, "pack_ent", [&] {
    k_pack_ent<<<grid_for(csr->nnz, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
        csr->col.p, csr->val32.p, csr->ent.p, csr->nnz);
  });
  if (csr->complex_h) {
    csr->val_im32.alloc(csr->nnz + kCsrPad);
    LEO_CUDA(cudaMemsetAsync(csr->val_im32.p + csr->nnz, 0, kCsrPad * sizeof(float), ctx->stream));
    launch(ctx, "to_f32", [&] {
      k_to_f32<<<grid_for(csr->nnz, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
          csr->val_im64.p, csr->val_im32.p, csr->nnz);
    });
  }
  if (csr->dx64.p) {
    csr->dx32.alloc(csr->nnz + kCsrPad);
    LEO_CUDA(cudaMemsetAsync(csr->dx32.p + csr->nnz, 0, kCsrPad * sizeof(float), ctx->stream));
    csr->entd.alloc(csr->nnz + kCsrPad);
    LEO_CUDA(cudaMemsetAsync(csr->entd.p + csr->nnz, 0, kCsrPad * sizeof(uint2), ctx->stream));
    launch(ctx, "to_f32", [&] {
      k_to_f32<<<grid_for(csr->nnz, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
          csr->dx64.p, csr->dx32.p, csr->nnz);
    });
    launch(ctx, "pack_ent", [&] {
      k_pack_ent<<<grid_for(csr->nnz, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
          csr->col.p, csr->dx32.p, csr->entd.p, csr->nnz);
    });
  }
}
}  // namespace leo2d

extern "C" leo2d_status leo2d_build_csr(leo2d_ctx* ctx, const leo2d_geom* g, uint32_t flags,
                                        leo2d_csr** out) {
  if (!ctx || !out) return LEO2D_ERR_BAD_ARG;
  *out = nullptr;
  leo2d_csr* csr = nullptr;
  leo2d_status st = guard(ctx, [&] {
    validate_geom(g);
    LEO_CUDA(cudaSetDevice(ctx->device));
    csr = new leo2d_csr();
    csr->device = ctx->device;
    csr->flags = flags;
    csr->geom = *g;
    csr->has_geom = true;
    GeomDev G;
    std::memset(&G, 0, sizeof(G));
    G.S = g->num_sheets;
    G.model = g->model;
    G.bc = g->boundary_condition;
    G.sc_search = g->boundary_condition == 1 ? g->sc_search_size : 0;
    G.keep_zeros = (flags & LEO2D_CSR_KEEP_ZEROS) ? 1 : 0;
    G.with_dx = (flags & LEO2D_CSR_WITH_DX) ? 1 : 0;
    G.b_field = g->b_field;
    G.kx = g->k_vec[0];
    G.ky = g->k_vec[1];
    G.cpx = (g->b_field != 0.0 || g->k_vec[0] != 0.0 || g->k_vec[1] != 0.0) ? 1 : 0;
    for (int s = 0; s < g->num_sheets; ++s)
      if (g->shifts[s][0] != 0.0 || g->shifts[s][1] != 0.0) G.shifted = 1;
    LEO_REQUIRE(!G.cpx || !G.with_dx,
                "the velocity operator (WITH_DX, conductivity) is not built for a complex Hamiltonian");
    std::memcpy(G.supercell, g->supercell, sizeof(G.supercell));
    G.rescale = g->energy_rescale;
    G.simple_amp = 0.33 / g->energy_rescale;
    G.shift = g->energy_shift;
    G.e_field = g->e_field;
    for (int r = 0; r <= kIntraShellMax; ++r) {
      const double raw = intra_shell_t(G.model, r);
      G.intra_q[r] = raw != 0.0 ? raw / G.rescale : 0.0;
    }
    G.diag_const = G.e_field == 0.0 ? 1 : 0;
    G.diag_q = (intra_shell_t(G.model, 0) + G.shift) / G.rescale;
    for (int s = 0; s < G.S; ++s) fill_sheet(*g, s, G.sh[s]);

    // sites of every sheet
    std::vector<DevBuf<int32_t>> grids(G.S), site_cells(G.S);
    int64_t n = 0;
    for (int s = 0; s < G.S; ++s) {
      SheetDev& d = G.sh[s];
      const int64_t cells = (int64_t)d.H * d.W * d.n_orb;
      DevBuf<int64_t> mask(cells), scan(cells + 1);
      launch(ctx, "site_mask", [&] {
        k_site_mask<<<grid_for(cells, 256, (int64_t)ctx->sm_count * 32), 256, 0, ctx->stream>>>(G, s, mask.p);
      });
      exclusive_scan_i64(ctx, mask.p, scan.p, cells);
      int64_t count = 0;
      d2h(ctx, &count, scan.p + cells, 1);
      ctx_sync(ctx);
      grids[s].alloc(cells);
      site_cells[s].alloc(count > 0 ? count : 1);
      launch(ctx, "site_fill", [&] {
        k_site_fill<<<grid_for(cells, 256, (int64_t)ctx->sm_count * 32), 256, 0, ctx->stream>>>(
            cells, mask.p, scan.p, grids[s].p, site_cells[s].p);
      });
      d.grid = grids[s].p;
      d.base = n;
      n += count;
      ctx_sync(ctx);
    }
    LEO_REQUIRE(n < (1ll << 31) - 1, "more than 2^31-1 orbitals: column indices are 32-bit");
    csr->n = n;
    csr->grid4.alloc(4 * (size_t)std::max<int64_t>(n, 1));
    csr->pos.alloc(3 * (size_t)std::max<int64_t>(n, 1));
    // a shifted job: the pairs from the unshifted positions (csr->pos during
    // assembly), the values from the shifted ones, which the matrix keeps
    DevBuf<double> spos_buf(G.shifted ? 3 * (size_t)std::max<int64_t>(n, 1) : 0);
    const double* spos = G.shifted ? spos_buf.p : csr->pos.p;
    DevBuf<const int32_t*> cell_ptrs(G.S);
    std::vector<const int32_t*> hp(G.S);
    for (int s = 0; s < G.S; ++s) hp[s] = site_cells[s].p;
    h2d(ctx, cell_ptrs.p, hp.data(), G.S);
    if (n > 0)
      launch(ctx, "sites", [&] {
        k_sites<<<grid_for(n, 256, (int64_t)ctx->sm_count * 32), 256, 0, ctx->stream>>>(
            G, n, cell_ptrs.p, csr->grid4.p, csr->pos.p, G.shifted ? spos_buf.p : nullptr);
      });

    // count -> scan -> fill
    DevBuf<int64_t> cnt_ent(std::max<int64_t>(n, 1)), cnt_intra(std::max<int64_t>(n, 1)),
        cnt_inter(std::max<int64_t>(n, 1));
    csr_alloc_rowptr(ctx, csr, n);
    RowOut ro{cnt_ent.p, cnt_intra.p, cnt_inter.p, csr->rowptr.p, nullptr, nullptr, nullptr, nullptr, nullptr};
    int cap = 0;
    size_t smem = 0;
    if (G.bc == 1) {
      const int n_img = (2 * G.sc_search + 1) * (2 * G.sc_search + 1);
      int neigh = (G.S > 1) ? (G.S > 2 ? 2 : 1) : 0;
      int need = n_img * ((2 * kIntraSearch) * (2 * kIntraSearch) * 2 +
                          neigh * (2 * kInterSearch) * (2 * kInterSearch) * 2);
      cap = 1;
      while (cap < need) cap <<= 1;
      smem = (size_t)cap * sizeof(uint64_t);
      LEO_REQUIRE(smem <= ctx->smem_optin, "periodic search too large for shared memory");
      LEO_CUDA(cudaFuncSetAttribute(k_periodic_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      LEO_CUDA(cudaFuncSetAttribute(k_periodic_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    const unsigned rows_grid = grid_for(n, kRowWarps, (int64_t)ctx->sm_count * 64);
    DevBuf<float4> pos32(G.bc == 0 ? std::max<int64_t>(n, 1) : 1);
    DevBuf<float4> spos32(G.bc == 0 && G.shifted ? std::max<int64_t>(n, 1) : 0);
    if (G.bc == 0 && n > 0)
      launch(ctx, "pos32", [&] {
        k_pos32<<<grid_for(n, 256, (int64_t)ctx->sm_count * 32), 256, 0, ctx->stream>>>(csr->pos.p, n, pos32.p);
        if (G.shifted)
          k_pos32<<<grid_for(n, 256, (int64_t)ctx->sm_count * 32), 256, 0, ctx->stream>>>(spos, n, spos32.p);
      });
    const float4* spos32p = G.shifted ? spos32.p : pos32.p;
    // the matrix keeps the job's (shifted) positions
    auto keep_shifted_positions = [&] {
      if (G.shifted) csr->pos = std::move(spos_buf);
    };
    const unsigned cta_grid = grid_for(n, 1, (int64_t)ctx->sm_count * 8);
    // A flake of the simple model without stored zeros (about 67 entries per
    // row) takes one pass: rows are filled into padded arrays of kPadCap
    // entries while they are counted, then compacted. A row with more entries,
    // or padded arrays too large for a quarter of free memory, takes the
    // count and fill passes.
    constexpr int kPadCap = 96;
    if (G.bc == 0 && n > 0 && G.model == LEO2D_MODEL_SIMPLE && !G.keep_zeros) {
      const size_t per = sizeof(int32_t) + sizeof(double) * (1 + (G.with_dx ? 2 : 0) + (G.cpx ? 1 : 0));
      size_t fr = 0, tot = 0;
      LEO_CUDA(cudaMemGetInfo(&fr, &tot));
      if ((size_t)n * kPadCap * per <= fr / 4) {
        const size_t pn = (size_t)n * kPadCap;
        DevBuf<int32_t> pcol(pn);
        DevBuf<double> pval(pn), pdx(G.with_dx ? pn : 0), pdy(G.with_dx ? pn : 0), pim(G.cpx ? pn : 0);
        DevBuf<int> overflow(1);
        LEO_CUDA(cudaMemsetAsync(overflow.p, 0, sizeof(int), ctx->stream));
        RowOut rp = ro;
        rp.col = pcol.p;
        rp.val = pval.p;
        rp.dx = pdx.p;
        rp.dy = pdy.p;
        rp.val_im = pim.p;
        rp.pad_cap = kPadCap;
        rp.overflow = overflow.p;
        launch(ctx, "flake_rows_fill", [&] {
          k_flake_rows<2><<<rows_grid, kRowWarps * 32, 0, ctx->stream>>>(G, n, csr->grid4.p, csr->pos.p, pos32.p, spos,
                                                              spos32p, rp);
        });
        int over = 0;
        d2h(ctx, &over, overflow.p, 1);
        ctx_sync(ctx);
        if (!over) {
          exclusive_scan_i64(ctx, cnt_ent.p, csr->rowptr.p, n);
          int64_t nnz = 0;
          d2h(ctx, &nnz, csr->rowptr.p + n, 1);
          ctx_sync(ctx);
          csr->nnz = nnz;
          csr->n_intra = reduce_sum_i64(ctx, cnt_intra.p, n);
          csr->n_inter = reduce_sum_i64(ctx, cnt_inter.p, n);
          csr_alloc_entries(ctx, csr, nnz, G.with_dx != 0);
          csr->complex_h = G.cpx != 0;
          if (csr->complex_h) {
            csr->val_im64.alloc(nnz + kCsrPad);
            LEO_CUDA(cudaMemsetAsync(csr->val_im64.p, 0, (nnz + kCsrPad) * sizeof(double), ctx->stream));
          }
          RowOut fo = ro;
          fo.col = csr->col.p;
          fo.val = csr->val64.p;
          fo.dx = csr->dx64.p;
          fo.dy = csr->dy64.p;
          fo.val_im = csr->val_im64.p;
          launch(ctx, "unpad_rows", [&] {
            k_unpad_rows<<<grid_for(n * 32, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
                n, kPadCap, csr->rowptr.p, pcol.p, pval.p, pdx.p, pdy.p, pim.p, fo);
          });
          ctx_check_status(ctx, "leo2d_build_csr (single pass)");
          keep_shifted_positions();
          csr_refresh_fp32(ctx, csr);
          ctx_sync(ctx);
          return;  // (the guard's lambda)
        }
      }
    }
    if (n > 0) {
      if (G.bc == 0)
        launch(ctx, "flake_rows_count", [&] {
          k_flake_rows<0><<<rows_grid, kRowWarps * 32, 0, ctx->stream>>>(G, n, csr->grid4.p, csr->pos.p, pos32.p, spos,
                                                              spos32p, ro);
        });
      else
        launch(ctx, "periodic_rows_count", [&] {
          k_periodic_rows<false><<<cta_grid, 256, smem, ctx->stream>>>(G, n, csr->grid4.p, csr->pos.p, spos,
                                                                       cap, ro, ctx->status.p);
        });
    }
    ctx_check_status(ctx, "leo2d_build_csr (count)");
    exclusive_scan_i64(ctx, cnt_ent.p, csr->rowptr.p, n);
    int64_t nnz = 0;
    d2h(ctx, &nnz, csr->rowptr.p + n, 1);
    ctx_sync(ctx);
    csr->nnz = nnz;
    csr->n_intra = reduce_sum_i64(ctx, cnt_intra.p, n);
    csr->n_inter = reduce_sum_i64(ctx, cnt_inter.p, n);
    csr_alloc_entries(ctx, csr, nnz, G.with_dx != 0);
    csr->complex_h = G.cpx != 0;
    csr->nonhermitian = csr->complex_h && G.bc == 1 && G.b_field != 0.0;
    if (csr->complex_h) {
      csr->val_im64.alloc(nnz + kCsrPad);
      LEO_CUDA(cudaMemsetAsync(csr->val_im64.p, 0, (nnz + kCsrPad) * sizeof(double), ctx->stream));
    }
    ro.col = csr->col.p;
    ro.val = csr->val64.p;
    ro.dx = csr->dx64.p;
    ro.dy = csr->dy64.p;
    ro.val_im = csr->val_im64.p;
    if (n > 0) {
      if (G.bc == 0)
        launch(ctx, "flake_rows_fill", [&] {
          k_flake_rows<1><<<rows_grid, kRowWarps * 32, 0, ctx->stream>>>(G, n, csr->grid4.p, csr->pos.p, pos32.p, spos,
                                                              spos32p, ro);
        });
      else
        launch(ctx, "periodic_rows_fill", [&] {
          k_periodic_rows<true><<<cta_grid, 256, smem, ctx->stream>>>(G, n, csr->grid4.p, csr->pos.p, spos,
                                                                      cap, ro, ctx->status.p);
        });
    }
    ctx_check_status(ctx, "leo2d_build_csr (fill)");
    keep_shifted_positions();
    csr_refresh_fp32(ctx, csr);
    ctx_sync(ctx);
  });
  if (st != LEO2D_OK) {
    delete csr;
    return st;
  }
  *out = csr;
  return LEO2D_OK;
}

namespace leo2d {

// Disregistry of every orbital into device memory out[n][2].
void csr_shift_configs(leo2d_ctx* ctx, const leo2d_csr* csr, double* out) {
  LEO_REQUIRE(csr->has_geom && csr->grid4.p, "matrix has no geometry (uploaded without it)");
  const leo2d_geom& g = csr->geom;
  LEO_REQUIRE(g.num_sheets == 2, "disregistry is defined for bilayers (two sheets)");
  GeomDev G;
  std::memset(&G, 0, sizeof(G));
  G.S = g.num_sheets;
  G.model = g.model;
  G.bc = g.boundary_condition;
  for (int s = 0; s < G.S; ++s) fill_sheet(g, s, G.sh[s]);
  CellInv ci;
  for (int s = 0; s < 2; ++s) {
    const double theta = g.angles[s];
    const SheetDev& d = G.sh[s];
    double u[2][2];
    u[0][0] = std::cos(theta) * d.a[0][0] - std::sin(theta) * d.a[0][1];
    u[0][1] = std::sin(theta) * d.a[0][0] + std::cos(theta) * d.a[0][1];
    u[1][0] = std::cos(theta) * d.a[1][0] - std::sin(theta) * d.a[1][1];
    u[1][1] = std::sin(theta) * d.a[1][0] + std::cos(theta) * d.a[1][1];
    const double det = u[0][0] * u[1][1] - u[0][1] * u[1][0];
    ci.inv[s][0][0] = u[1][1] / det;
    ci.inv[s][0][1] = -u[1][0] / det;
    ci.inv[s][1][0] = -u[0][1] / det;
    ci.inv[s][1][1] = u[0][0] / det;
  }
  if (csr->n > 0)
    launch(ctx, "shift_configs", [&] {
      k_shift_configs<<<grid_for(csr->n, 256, (int64_t)ctx->sm_count * 16), 256, 0, ctx->stream>>>(
          G, ci, csr->n, csr->grid4.p, out);
    });
}

}  // namespace leo2d

extern "C" leo2d_status leo2d_csr_shift_configs(leo2d_ctx* ctx, const leo2d_csr* csr, double* out) {
  if (!ctx || !csr || !out) return LEO2D_ERR_BAD_ARG;
  return guard(ctx, [&] {
    LEO_CUDA(cudaSetDevice(ctx->device));
    DevBuf<double> d(2 * (size_t)std::max<int64_t>(csr->n, 1));
    csr_shift_configs(ctx, csr, d.p);
    d2h(ctx, out, d.p, 2 * (size_t)csr->n);
    ctx_sync(ctx);
  });
}
