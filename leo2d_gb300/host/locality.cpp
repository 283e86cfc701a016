// locality.cpp - the job driver of the KPM path, host side.
//
// Replaces, for one process on one GPU, what the reference spreads over an MPI
// job farm: Locality::constructGeom (src/locality.cpp:785-1187),
// rootChebSolve's job and trace-vector set-up (1271-2320) and the worker block
// of workerChebSolve (3041-3148): geometry and H~ are built on the GPU
// (leo2d_build_csr), the recursion runs there (leo2d_kpm_dos / _ldos / _cond),
// the transforms run there (leo2d_dos_transform / leo2d_cond_transform), and
// the files are written as Param_tools::save (src/params/param_tools.cpp:19-316)
// and generateRealH (src/locality.cpp:4366-4448) write them.
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <random>
#include <sstream>

#include "job.h"

namespace leo2d_host {

namespace {

struct Ctx {
  leo2d_ctx* h = nullptr;
  ~Ctx() {
    if (h) leo2d_ctx_destroy(h);
  }
};
struct Csr {
  leo2d_csr* h = nullptr;
  ~Csr() {
    if (h) leo2d_csr_destroy(h);
  }
};

#define CHECK(call)                                                         \
  do {                                                                      \
    leo2d_status st_ = (call);                                              \
    if (st_ != LEO2D_OK) {                                                  \
      err = std::string(#call) + ": " + leo2d_last_error(ctx.h);            \
      return st_;                                                           \
    }                                                                       \
  } while (0)

std::string join_path(const std::string& dir, const std::string& name) {
  if (dir.empty() || dir == ".") return name;
  return dir.back() == '/' ? dir + name : dir + "/" + name;
}

// Hstruct::getTargetList, solver type SQ (src/geom/hstruct.cpp:1056-1079):
// the orbitals of the grid-centre cell of each target sheet.
bool target_list(const JobSpec& spec, const std::vector<int32_t>& grid4, std::vector<int64_t>& out,
                 std::string& err) {
  const leo2d_geom& g = spec.geom;
  const int64_t n = (int64_t)grid4.size() / 4;
  for (int ts : spec.target_sheets) {
    if (ts < 0 || ts >= g.num_sheets) {
      err = "TARGET_SHEETS names a sheet that does not exist";
      return false;
    }
    const int x_off = (g.max_shape[ts][0] - g.min_shape[ts][0]) / 2;
    const int y_off = (g.max_shape[ts][1] - g.min_shape[ts][1]) / 2;
    int64_t center = -1;
    for (int64_t k = 0; k < n; ++k)
      if (grid4[4 * k] == x_off && grid4[4 * k + 1] == y_off && grid4[4 * k + 2] == 0 &&
          grid4[4 * k + 3] == ts) {
        center = k;
        break;
      }
    if (center < 0) {
      err = "the centre cell of target sheet " + std::to_string(ts + 1) + " holds no orbital";
      return false;
    }
    for (int orb = 0; orb < 2; ++orb) out.push_back(center + orb);
  }
  return true;
}

void write_energies(std::ofstream& f, const std::vector<double>& E) {
  for (double e : E) f << e << " ";
  f << "\n";
}

// One job of the vacancy solvers: its vacancies (0-based) and targets, and for
// MLMC_VAC its IDs from the vacancy file.
struct VacJob {
  std::vector<int64_t> vacancies;
  std::vector<int64_t> targets;
  int mlmc_id = -1, cluster_id = -1;
};

// Locality::getVacanciesFromFile (src/locality.cpp:536-640). MLMC_VAC: lines
// "JOBID = j", "CLUSTERID = c" and "VAC = v1,v2,..." (1-based, no spaces in the
// list), a job per JOBID; the IDs (j, c) are also the job's target list
// (locality.cpp:1432-1446), and a list that is just "-1" means no vacancies.
// VD_FILE: the file vacancies.dat, each "JOB=" line followed by a line of
// vacancies and a line of targets (1-based, comma-separated).
bool read_vacancy_jobs(int solver_type, const std::string& path, std::vector<VacJob>& jobs, std::string& err) {
  std::ifstream in(path);
  if (!in.is_open()) {
    err = "cannot read the vacancy file " + path;
    return false;
  }
  std::string line;
  if (solver_type == 3) {
    int job_id = -1, cluster_id = -1;
    std::vector<int64_t> vac;
    auto push = [&]() {
      VacJob j;
      j.vacancies = vac;
      // "VAC = -1" (read as -2): the job has no vacancies (locality.cpp:1425-1430)
      if (j.vacancies.size() == 1 && j.vacancies[0] == -2) j.vacancies.clear();
      j.targets = {job_id, cluster_id};
      j.mlmc_id = job_id;
      j.cluster_id = cluster_id;
      jobs.push_back(j);
      vac.clear();
    };
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::string tok;
      while (std::getline(ls, tok, ' ')) {
        if (tok == "JOBID") {
          if (job_id != -1) push();
          std::getline(ls, tok, ' ');
          std::getline(ls, tok, ' ');
          job_id = std::atoi(tok.c_str());
        } else if (tok == "CLUSTERID") {
          std::getline(ls, tok, ' ');
          std::getline(ls, tok, ' ');
          cluster_id = std::atoi(tok.c_str());
        } else if (tok == "VAC") {
          std::getline(ls, tok, ' ');
          std::string list;
          std::getline(ls, list, ' ');
          std::istringstream vs(list);
          while (std::getline(vs, tok, ',')) vac.push_back(std::atoi(tok.c_str()) - 1);
        }
      }
    }
    push();  // the last job
  } else {
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::string tok;
      while (std::getline(ls, tok, '=')) {
        if (tok != "JOB") continue;
        std::string vline, tline;
        std::getline(in, vline);
        std::getline(in, tline);
        VacJob j;
        std::istringstream vs(vline), ts(tline);
        while (std::getline(vs, tok, ',')) j.vacancies.push_back(std::atoi(tok.c_str()) - 1);
        while (std::getline(ts, tok, ',')) j.targets.push_back(std::atoi(tok.c_str()) - 1);
        jobs.push_back(j);
      }
    }
  }
  if (jobs.empty()) {
    err = "the vacancy file " + path + " holds no job";
    return false;
  }
  return true;
}

// Mlmc_handler (src/mlmc/mlmc_handler.cpp) for trace-DOS jobs: running means
// of the jobs' DOS (E) and of its square (V), and for jobs of a cluster the
// same of the difference from the cluster's original at the next level (DE,
// DV), with Param_tools::mlmc_average / _variance / _cluster_average /
// _cluster_variance's update (param_tools.cpp:1213-1720): with c the
// accumulator's sample count, x <- x (c - 1) / c + sample / c, the first sample
// taken as is. Files as Param_tools::mlmc_save / mlmc_load (975-1211): raw FP64.
struct MlmcStats {
  std::vector<double> E, V, DE, DV;
  int nE = 1, nV = 1, nDE = 1, nDV = 1;
  std::vector<std::vector<double>> cluster_original;

  static void update(std::vector<double>& tot, int& count, const std::vector<double>& samp) {
    if (tot.empty() || count == 1) {
      tot = samp;
    } else {
      const double s_t = (1.0 * count - 1) / (1.0 * count), s_s = 1.0 / (1.0 * count);
      for (size_t i = 0; i < tot.size() && i < samp.size(); ++i) tot[i] = tot[i] * s_t + samp[i] * s_s;
    }
    ++count;
  }
  static std::vector<double> square(const std::vector<double>& x) {
    std::vector<double> y(x.size());
    for (size_t i = 0; i < x.size(); ++i) y[i] = std::pow(x[i], 2);
    return y;
  }
  static std::vector<double> diff(const std::vector<double>& a, const std::vector<double>& b) {
    std::vector<double> y(a.size());
    for (size_t i = 0; i < a.size(); ++i) y[i] = a[i] - (i < b.size() ? b[i] : 0.0);
    return y;
  }
  static std::vector<double> load(const std::string& file) {
    std::ifstream f(file, std::ios::binary | std::ios::ate);
    if (!f.is_open()) return {};
    const std::streamsize bytes = f.tellg();
    std::vector<double> v((size_t)std::max<std::streamsize>(bytes, 0) / sizeof(double));
    f.seekg(0);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(v.size() * sizeof(double)));
    return v;
  }
  static bool save(const std::string& file, const std::vector<double>& v) {
    std::ofstream f(file, std::ios::binary);
    if (!f.is_open()) return false;
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(double)));
    return true;
  }
};

std::string mlmc_name(const std::string& root, const std::string& prefix, int level, const std::string& tail) {
  return root + "/" + prefix + "_L" + std::to_string(level) + tail;
}

}  // namespace

leo2d_status run_job(const JobSpec& spec, const std::string& out_dir, int device, std::string& err) {
  if (!spec.unsupported.empty()) {
    err = "options outside this build's KPM path:";
    for (const auto& u : spec.unsupported) err += " [" + u + "]";
    return LEO2D_ERR_UNSUPPORTED;
  }
  const int P = spec.poly_order;
  if (P % 4 != 0 || P < 4) {  // main.cpp:914-917
    err = "poly_order = " + std::to_string(P) + " is NOT divisible 4 (needed for KPM iterative method)";
    return LEO2D_ERR_BAD_ARG;
  }
  if (spec.solver_type < 1 || spec.solver_type > 6 || spec.solver_type == 5) {
    err = "SOLVER_TYPE must be SQ, LC, MLMC_VAC, VD_FILE or FIXED_SHIFT (their job lists are built)";
    return LEO2D_ERR_UNSUPPORTED;
  }
  if (spec.mlmc == 1 && spec.solver_type != 3) {
    err = "MLMC = 1 takes its jobs from SOLVER_TYPE = MLMC_VAC";
    return LEO2D_ERR_BAD_ARG;
  }
  if ((spec.solver_type == 3 || spec.solver_type == 4) &&
      (spec.geom.boundary_condition != 0 || spec.use_b == 1 || spec.k_sampling == 1 || spec.observable_type != 0)) {
    err = "the vacancy solvers run DOS jobs on real flakes here (no periodic cell, field, k points or COND)";
    return LEO2D_ERR_UNSUPPORTED;
  }
  if (spec.solver_type == 2 && (spec.num_lc_points < 2 || spec.lc_points.size() < 2 * (size_t)spec.num_lc_points)) {
    err = "SOLVER_TYPE = LC needs NUM_LC_POINTS >= 2 and its LC_POINTS";
    return LEO2D_ERR_BAD_ARG;
  }
  if (spec.k_sampling == 1 && spec.k_type == 1 && spec.geom.num_sheets < 2) {  // locality.cpp:1661-1663
    err = "cannot use K_TYPE == 1 (twisted BZ) for a single layer";
    return LEO2D_ERR_BAD_ARG;
  }
  if (spec.k_sampling == 1 && spec.k_type == 4 &&
      (spec.geom.boundary_condition != 1 || spec.geom.num_sheets != 2 ||
       (spec.geom.supercell_m == 0 && spec.geom.supercell_n == 0))) {
    // locality.cpp:1996-2039: the zone of the bilayer (M, N) supercell. The
    // trilayer's cell [0 q; -q q] puts M on the y axis, where the reference's
    // M -> Gamma leg divides by zero: its k points there are NaN.
    err = spec.geom.num_sheets == 3
              ? "K_TYPE = 4 on a trilayer: the reference's M -> Gamma leg divides by zero there (NaN k points)"
              : "K_TYPE = 4 samples the zone of a bilayer SUPERCELL_M_N supercell";
    return LEO2D_ERR_UNSUPPORTED;
  }
  if (spec.k_sampling == 1 && spec.k_type == 5 &&
      (spec.geom.boundary_condition != 1 || spec.geom.num_sheets != 3)) {
    // locality.cpp:2161-2182: the K points of the three layers
    err = "K_TYPE = 5 joins the K points of a trilayer supercell's three sheets";
    return LEO2D_ERR_UNSUPPORTED;
  }
  if (spec.k_sampling == 1 && (spec.num_k1 < 1 || (spec.k_type == 0 && spec.num_k2 < 1))) {
    err = "K_GRID must name at least one k point";
    return LEO2D_ERR_BAD_ARG;
  }
  if (spec.nshifts < 1) {
    err = "NSHIFTS must be >= 1";
    return LEO2D_ERR_BAD_ARG;
  }
  for (int s : spec.shift_sheets)
    if (s < 0 || s >= spec.geom.num_sheets) {
      err = "SHIFT_SHEETS names a sheet that does not exist";
      return LEO2D_ERR_BAD_ARG;
    }
  if (spec.nshifts > 1 && (int)spec.shift_sheets.size() < spec.num_shift_sheets) {
    err = "NSHIFTS > 1 needs SHIFT_SHEETS for its NUM_SHIFT_SHEETS sheets";
    return LEO2D_ERR_BAD_ARG;
  }
  Ctx ctx;
  {
    leo2d_status st = leo2d_ctx_create(&ctx.h, device);
    if (st != LEO2D_OK) {
      err = "no usable CUDA device";
      return st;
    }
  }
  leo2d_geom g0 = spec.geom;
  CHECK(leo2d_geom_prepare(&g0));
  // the job list of the SQ solver (recursiveShiftCalc, locality.cpp:1222-1269):
  // for the last shift sheet every (i/N, j/N), i outer, j inner, and for each
  // of those the list of the remaining shift sheets
  std::vector<std::vector<double>> jobs;  // [job][2 * sheet]
  std::vector<VacJob> vjobs;              // the vacancy solvers' jobs (no shifts)
  if (spec.solver_type == 3 || spec.solver_type == 4) {
    // MLMC_VAC reads VACANCY_FILE; VD_FILE reads vacancies.dat (locality.cpp:536, 591)
    // (relative paths: in the output directory, the reference's working directory)
    std::string vf = spec.solver_type == 3 ? spec.vacancy_file : std::string("vacancies.dat");
    if (!vf.empty() && vf[0] != '/') vf = join_path(out_dir, vf);
    if (!read_vacancy_jobs(spec.solver_type, vf, vjobs, err)) return LEO2D_ERR_IO;
    // VD_FILE jobs never set num_vacancies, so the worker removes nothing (locality.cpp:1456-1494, 2994)
    if (spec.solver_type == 4)
      for (auto& j : vjobs) j.vacancies.clear();
    for (size_t i = 0; i < vjobs.size(); ++i) jobs.push_back(std::vector<double>(2 * LEO2D_MAX_SHEETS, 0.0));
  } else if (spec.solver_type == 6) {
    // one job, every sheet but the first shifted by (1/3, 1/3) (locality.cpp:1580-1608)
    std::vector<double> sh(2 * LEO2D_MAX_SHEETS, 0.0);
    for (int s = 1; s < g0.num_sheets; ++s) sh[2 * s] = sh[2 * s + 1] = 1.0 / 3.0;
    jobs.push_back(sh);
  } else if (spec.solver_type == 2) {
    // line cuts (locality.cpp:1330-1386): NSHIFTS jobs along the polyline of
    // LC_POINTS, each shifting the last sheet
    const int nj = spec.nshifts, m = spec.num_lc_points;
    const int last = g0.num_sheets - 1;
    for (int i = 0; i < nj; ++i) {
      const double x = (1.0 / ((double)nj)) * i;
      const double total_x = x * (m - 1);
      const int idx = (int)std::floor(total_x);
      const double eff_x = std::fmod(total_x, 1);
      const double* a = &spec.lc_points[2 * (size_t)idx];
      const double* b = &spec.lc_points[2 * (size_t)std::min(idx + 1, m - 1)];
      std::vector<double> sh(2 * LEO2D_MAX_SHEETS, 0.0);
      sh[2 * last] = a[0] + eff_x * (b[0] - a[0]);
      sh[2 * last + 1] = a[1] + eff_x * (b[1] - a[1]);
      std::printf("shifts[%d] = [%lf %lf] \n", last, sh[2 * last], sh[2 * last + 1]);
      jobs.push_back(sh);
    }
  } else {
    std::vector<double> sh(2 * LEO2D_MAX_SHEETS, 0.0);
    const int levels = spec.nshifts > 1 ? spec.num_shift_sheets : 0;
    const int N = spec.nshifts;
    auto rec = [&](auto&& self, int k) -> void {
      if (k == 0) {
        jobs.push_back(sh);
        return;
      }
      const int tar = spec.shift_sheets[k - 1];
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
          sh[2 * tar] = (1.0 / (double)(N)) * i;
          sh[2 * tar + 1] = (1.0 / (double)(N)) * j;
          self(self, k - 1);
        }
    };
    rec(rec, levels);
  }
  // K_SAMPLING with K_TYPE = 0 (locality.cpp:1615-1650): each job at every
  // point k = (k1/n1) b1 + (k2/n2) b2 of the supercell's reciprocal grid, k1
  // outer, k2 inner; b from Locality::getReciprocal (locality.cpp:7215-7262)
  std::vector<std::array<double, 2>> kjobs;
  if (spec.k_sampling == 1) {
    auto reciprocal = [](const double (&a2)[2][2], double (&b)[2][2]) {
      const double a[3][3] = {{a2[0][0], a2[0][1], 0.0}, {a2[1][0], a2[1][1], 0.0}, {0.0, 0.0, 1.0}};
      auto cross = [](const double* x, const double* y, int d) {
        return d == 0 ? x[1] * y[2] - x[2] * y[1] : (d == 1 ? x[2] * y[0] - x[0] * y[2] : x[0] * y[1] - x[1] * y[0]);
      };
      double den1 = 0.0, den2 = 0.0;
      for (int j = 0; j < 3; ++j) {
        den1 += a[0][j] * cross(a[1], a[2], j);
        den2 += a[1][j] * cross(a[2], a[0], j);
      }
      for (int k = 0; k < 2; ++k) {
        b[0][k] = 2 * M_PI * cross(a[1], a[2], k) / den1;
        b[1][k] = 2 * M_PI * cross(a[2], a[0], k) / den2;
      }
    };
    // Locality::getReciprocal(int) (locality.cpp:7168-7213): sheet s's lattice
    // turned by its angle
    auto sheet_reciprocal = [&](int s, double (&bs)[2][2]) {
      double as[2][2];
      const double th = g0.angles[s];
      for (int i = 0; i < 2; ++i) {
        as[i][0] = g0.lattice[s][i][0] * std::cos(th) - g0.lattice[s][i][1] * std::sin(th);
        as[i][1] = g0.lattice[s][i][0] * std::sin(th) + g0.lattice[s][i][1] * std::cos(th);
      }
      reciprocal(as, bs);
    };
    double b[2][2];
    reciprocal(g0.supercell, b);
    std::vector<std::vector<double>> shift_jobs = jobs;
    jobs.clear();
    if (spec.k_type == 4) {
      // K_TYPE 4 (locality.cpp:1990-2159): 3 NUM_K1 points of the bilayer (M, N)
      // supercell's zone, Gamma -> K -> M -> Gamma. The zone is that of the
      // cell A = [N M; -M M+N] (M > N) or [M N; -N M+N] in sheet 0's unrotated
      // lattice vectors; M = (b1 + b2) / 2, K = b2 turned by +30 degrees over
      // sqrt 3. Each leg is walked by the reference's slope and intercept, with
      // its operations in its order: the second leg adds no intercept, and the
      // third runs along y from M when M's two coordinates are equal.
      const int Mi = g0.supercell_m, Ni = g0.supercell_n;
      const int A11 = Mi > Ni ? Ni : Mi, A12 = Mi > Ni ? Mi : Ni;
      const int A21 = Mi > Ni ? -Mi : -Ni, A22 = Mi + Ni;
      const auto& a0 = g0.lattice[0];
      const double sc4[2][2] = {{A11 * a0[0][0] + A12 * a0[1][0], A11 * a0[0][1] + A12 * a0[1][1]},
                                {A21 * a0[0][0] + A22 * a0[1][0], A21 * a0[0][1] + A22 * a0[1][1]}};
      double bs[2][2];
      reciprocal(sc4, bs);
      const double r3 = std::sqrt(3.0), alpha = M_PI / 6;
      const double rot30[2][2] = {{std::cos(alpha), std::sin(alpha)}, {-std::sin(alpha), std::cos(alpha)}};
      const double gm[2] = {0.0, 0.0};
      double mm[2], kk[2];
      for (int i = 0; i < 2; ++i) mm[i] = 0.5 * (bs[0][i] + bs[1][i]);
      for (int i = 0; i < 2; ++i) {
        kk[i] = 0;
        for (int j = 0; j < 2; ++j) kk[i] = kk[i] + rot30[i][j] * bs[1][j] / r3;
      }
      const double s1 = (kk[1] - gm[1]) / (kk[0] - gm[0]);
      const double s2 = (mm[1] - kk[1]) / (mm[0] - kk[0]);
      const double s3 = (gm[1] - mm[1]) / (gm[0] - mm[0]);
      const double c1 = (kk[0] * gm[1] - gm[0] * kk[1]) / (kk[0] - gm[0]);
      const double c3 = (gm[0] * mm[1] - mm[0] * gm[1]) / (gm[0] - mm[0]);
      const double l1 = kk[0] - gm[0], l2 = mm[0] - kk[0], l3 = gm[0] - mm[0];
      const int nk = spec.num_k1;
      for (const auto& sj : shift_jobs)
        for (int i = 0; i < 3 * nk; ++i) {
          double kx, ky;
          if (i < nk) {
            kx = gm[0] + i * l1 / nk;
            ky = gm[1] + s1 * i * l1 / nk + c1;
          } else if (i < 2 * nk) {
            const int n2 = i - nk;
            kx = kk[0] + n2 * l2 / nk;
            ky = kk[1] + s2 * n2 * l2 / nk;
          } else {
            const int n3 = i - 2 * nk;
            if (mm[0] == mm[1]) {
              const double len = gm[1] - mm[1];
              kx = mm[0];
              ky = mm[1] + n3 * len / nk;
            } else {
              kx = mm[0] + n3 * l3 / nk;
              ky = mm[1] + s3 * n3 * l3 / nk + c3;
            }
          }
          jobs.push_back(sj);
          kjobs.push_back({kx, ky});
        }
    } else if (spec.k_type == 5) {
      // K_TYPE 5 (locality.cpp:2161-2250): the path through the K points of the
      // three layers, K_s = (2 b_s1 + b_s2) / 3 with b_s the reciprocal vectors
      // of sheet s's lattice turned by its angle: NUM_K1 points from K_0 to K_1,
      // NUM_K1 from K_1 to K_2 (each on its line's slope and intercept), then K_2.
      double kl[3][2];
      for (int s3 = 0; s3 < 3; ++s3) {
        double bs[2][2];
        sheet_reciprocal(s3, bs);
        for (int i = 0; i < 2; ++i) kl[s3][i] = 1.0 / 3.0 * (2.0 * bs[0][i] + bs[1][i]);
      }
      const double s1 = (kl[1][1] - kl[0][1]) / (kl[1][0] - kl[0][0]);
      const double s2 = (kl[2][1] - kl[1][1]) / (kl[2][0] - kl[1][0]);
      const double m1 = kl[1][1] - s1 * kl[1][0];
      const double m2 = kl[2][1] - s2 * kl[2][0];
      const double l1 = kl[1][0] - kl[0][0], l2 = kl[2][0] - kl[1][0];
      const int nk = spec.num_k1, last = 2 * nk;
      for (const auto& sj : shift_jobs)
        for (int i = 0; i < last + 1; ++i) {
          double kx, ky;
          if (i < nk) {
            kx = kl[0][0] + i * l1 / nk;
            ky = s1 * kx + m1;
          } else if (i < last) {
            const int n2 = i - nk;
            kx = kl[1][0] + n2 * l2 / nk;
            ky = s2 * kx + m2;
          } else {
            kx = kl[2][0];
            ky = kl[2][1];
          }
          jobs.push_back(sj);
          kjobs.push_back({kx, ky});
        }
    } else if (spec.k_type >= 1) {
      // k paths (locality.cpp:1655-1990): each job at NUM_K1 points of a path through
      // the corners P_0 .. P_L; point i sits at c = L i / NUM_K1 and on leg j = the
      // first with c <= j + 1 (the last leg takes the rest), at (j+1-c) P_j + (c-j) P_j+1.
      //   K_TYPE 1: supercell zone, K -> Gamma -> M -> K
      //   K_TYPE 2: sheet 0's own zone, Gamma -> M -> K -> Gamma
      //   K_TYPE 3: supercell zone, Gamma -> M -> K -> K' -> Gamma
      // Supercell zone: K = b2 turned by -30 degrees over 2 cos 30, K' = K turned by
      // -60 degrees, M = b2 / 2. Sheet 0's zone: b1 from its lattice turned by its
      // angle (Locality::getReciprocal(int), locality.cpp:7168-7213), M = b1[0] / 2,
      // K = M turned by 30 degrees over cos 30.
      using Pt = std::array<double, 2>;
      const Pt gm = {0.0, 0.0};
      std::vector<Pt> pts;
      if (spec.k_type == 2) {
        double b1[2][2];
        sheet_reciprocal(0, b1);
        const double h = (M_PI / 3.0) / 2.0;
        const Pt mm = {b1[0][0] / 2.0, b1[0][1] / 2.0};
        const Pt kk = {(mm[0] * std::cos(h) - mm[1] * std::sin(h)) / std::cos(h),
                       (mm[0] * std::sin(h) + mm[1] * std::cos(h)) / std::cos(h)};
        pts = {gm, mm, kk, gm};
      } else {
        const double r = 1.0 / (2.0 * std::cos(M_PI / 6));
        const Pt kk = {r * (std::cos(-M_PI / 6) * b[1][0] - std::sin(-M_PI / 6) * b[1][1]),
                       r * (std::sin(-M_PI / 6) * b[1][0] + std::cos(-M_PI / 6) * b[1][1])};
        const Pt mm = {b[1][0] / 2.0, b[1][1] / 2.0};
        if (spec.k_type == 1) {
          pts = {kk, gm, mm, kk};
        } else {
          const Pt k2 = {std::cos(-M_PI / 3) * kk[0] - std::sin(-M_PI / 3) * kk[1],
                         std::sin(-M_PI / 3) * kk[0] + std::cos(-M_PI / 3) * kk[1]};
          pts = {gm, mm, kk, k2, gm};
        }
      }
      const int legs = (int)pts.size() - 1;
      for (const auto& sj : shift_jobs)
        for (int i = 0; i < spec.num_k1; ++i) {
          const double c = ((double)legs / (double)spec.num_k1) * i;
          int j = 0;
          while (j < legs - 1 && c > j + 1) ++j;
          Pt k;
          for (int d = 0; d < 2; ++d) k[d] = ((j + 1.0) - c) * pts[j][d] + (c - j) * pts[j + 1][d];
          jobs.push_back(sj);
          kjobs.push_back(k);
        }
    }
    for (const auto& sj : spec.k_type == 0 ? shift_jobs : std::vector<std::vector<double>>())
      for (int k1 = 0; k1 < spec.num_k1; ++k1)
        for (int k2 = 0; k2 < spec.num_k2; ++k2) {
          jobs.push_back(sj);
          kjobs.push_back({(k1 / (double)spec.num_k1) * b[0][0] + (k2 / (double)spec.num_k2) * b[1][0],
                           (k1 / (double)spec.num_k1) * b[0][1] + (k2 / (double)spec.num_k2) * b[1][1]});
        }
  }
  // a complex Hamiltonian: a magnetic field or Bloch phases (locality.cpp:2906-2909)
  const bool cpx_run = spec.use_b == 1 || spec.k_sampling == 1;
  const bool gersh = spec.bounds == 1;
  uint32_t flags = 0;
  if (spec.observable_type == 1 || spec.matrix_save > 1) flags |= LEO2D_CSR_WITH_DX;
  // generateCpxH's matrix save lists every stored pair, zeros included (locality.cpp:5213-5228)
  if (cpx_run && spec.matrix_save > 0) flags |= LEO2D_CSR_KEEP_ZEROS;
  // (an MLMC run writes its level statistics instead of a .cheb, locality.cpp:2773-2837)
  std::ofstream cheb;
  if (spec.mlmc != 1) {
    cheb.open(join_path(out_dir, spec.job_name + ".cheb"));
    if (!cheb.is_open()) {
      err = "cannot write " + spec.job_name + ".cheb";
      return LEO2D_ERR_IO;
    }
  }
  cheb << std::fixed;
  // Mlmc_handler::setup (mlmc_handler.cpp:29-116): below the top level, the
  // cluster originals are the next level's saved job results
  MlmcStats mlmc;
  const std::string mlmc_out = spec.mlmc_out_root.empty() || spec.mlmc_out_root[0] == '/'
                                   ? spec.mlmc_out_root : join_path(out_dir, spec.mlmc_out_root);
  const std::string mlmc_temp = spec.mlmc_temp_root.empty() || spec.mlmc_temp_root[0] == '/'
                                    ? spec.mlmc_temp_root : join_path(out_dir, spec.mlmc_temp_root);
  if (spec.mlmc == 1 && spec.mlmc_level < spec.mlmc_max_level)
    for (int i = 0; i < spec.mlmc_num_clusters; ++i)
      mlmc.cluster_original.push_back(spec.kpm_trace == 1
                                          ? MlmcStats::load(mlmc_name(mlmc_temp, spec.job_name, spec.mlmc_level + 1,
                                                                      "_J" + std::to_string(i + 1) + "_dos.bin"))
                                          : std::vector<double>());
  // one generator draws every job's trace vectors in job order (locality.cpp:2274-2305)
  std::default_random_engine generator;
  std::normal_distribution<double> distribution(0.0, 1.0);
  Csr csr;
  int64_t n = 0, nnz = 0;
  std::vector<int32_t> grid4;
  std::vector<double> pos;
  std::vector<int64_t> targets;
  bool last_complex = false;
  for (size_t job = 0; job < jobs.size(); ++job) {
    const bool first_job = job == 0;
    leo2d_geom g = g0;
    for (int s = 0; s < g.num_sheets; ++s) {
      g.shifts[s][0] = jobs[job][2 * s];
      g.shifts[s][1] = jobs[job][2 * s + 1];
    }
    if (!kjobs.empty()) {
      g.k_vec[0] = kjobs[job][0];
      g.k_vec[1] = kjobs[job][1];
    }
    last_complex = g.b_field != 0.0 || g.k_vec[0] != 0.0 || g.k_vec[1] != 0.0;
    double rescale = g.energy_rescale, shift = g.energy_shift, center = -shift;
    if (gersh) {
      g.energy_rescale = 1.0;
      g.energy_shift = 0.0;
    }
    if (csr.h) {
      leo2d_csr_destroy(csr.h);
      csr.h = nullptr;
    }
    CHECK(leo2d_build_csr(ctx.h, &g, flags, &csr.h));
    int64_t ni = 0, ne = 0;
    CHECK(leo2d_csr_info(csr.h, &n, &nnz, &ni, &ne));
    if (first_job)  // constructGeom reports the geometry once
      std::printf("Heterostructure has %lld orbitals. \n%lld entries expected from intra. \n"
                  "%lld entries expected from inter. \n",
                  (long long)n, (long long)ni, (long long)ne);
    if (gersh) {
      double lo = 0, hi = 0;
      CHECK(leo2d_csr_bounds(ctx.h, csr.h, &lo, &hi));
      rescale = 1.01 * (hi - lo) / 2;
      center = (hi + lo) / 2;
      shift = -center;
      CHECK(leo2d_csr_rescale(ctx.h, csr.h, rescale, shift));
    }
    grid4.assign(4 * n, 0);
    pos.assign(3 * n, 0.0);
    CHECK(leo2d_csr_geometry(ctx.h, csr.h, grid4.data(), pos.data()));
    if (vjobs.empty() && first_job && !target_list(spec, grid4, targets, err)) return LEO2D_ERR_BAD_ARG;
    // the vacancy solvers: the job's own targets, and its matrix without its
    // vacancies (workerChebSolve, locality.cpp:2989-3016)
    Csr vcsr;
    leo2d_csr* kcsr = csr.h;
    int64_t n_kpm = n;
    int n_vac = 0;
    if (!vjobs.empty()) {
      const VacJob& vj = vjobs[job];
      n_vac = (int)vj.vacancies.size();
      if (n_vac > 0) {
        CHECK(leo2d_csr_remove_orbitals(ctx.h, csr.h, vj.vacancies.data(), (int64_t)n_vac, &vcsr.h));
        int64_t z0 = 0, z1 = 0, z2 = 0;
        CHECK(leo2d_csr_info(vcsr.h, &n_kpm, &z0, &z1, &z2));
        kcsr = vcsr.h;
        // the root draws trace vectors of max_index - num_vacancies entries
        // (locality.cpp:2282-2287): a list with repeats or orbitals outside the
        // flake would not match the worker's matrix
        if (n - n_kpm != n_vac) {
          err = "vacancy list of job " + std::to_string(job + 1) + " repeats orbitals or names ones outside the flake";
          return LEO2D_ERR_BAD_ARG;
        }
      }
      targets.clear();
      for (int64_t t : vj.targets) {
        int64_t below = 0;
        for (int64_t v : vj.vacancies) below += v < t ? 1 : 0;
        targets.push_back(t - below);
      }
    }

    // Chebyshev nodes of Param_tools::save (param_tools.cpp:57-62); with
    // Gershgorin bounds the axis is centre + rescale x.
    std::vector<double> E(P);
    for (int i = 0; i < P; ++i) {
      const double x = std::cos((i * 1.0 + 0.5) * M_PI / P);
      E[i] = gersh ? center + rescale * x : shift + rescale * x;
    }

    // (the sheet and target lines are written for the SQ and LC solvers only)
    if (spec.verbose_save != 0) cheb << "JOBID = " << job + 1 << " \n";
    if (spec.verbose_save != 0 && spec.solver_type != 6) {  // Param_tools::saveHeader (param_tools.cpp:467-505)
      cheb << "SHEET: SHIFT_X, SHIFT_Y, SHIFT_Z \n";
      for (int s = 0; s < g.num_sheets; ++s)
        cheb << s + 1 << "    : " << g.shifts[s][0] << ", " << g.shifts[s][1] << ", " << 0.0 << " \n";
      cheb << "NUM_TAR = " << targets.size() << "\n";
      if (!targets.empty()) {
        cheb << "TAR_LIST: ";
        for (size_t t = 0; t + 1 < targets.size(); ++t) cheb << targets[t] << ", ";
        cheb << targets.back() << " \n";
      } else {
        cheb << "NO_TAR \n";
      }
    }
    if (spec.verbose_save != 0 && (spec.use_b == 1 || spec.use_e == 1)) {  // param_tools.cpp:572-575
      cheb << "MAG_ON  = " << spec.use_b << ", B = " << spec.b_field << " \n";
      cheb << "ELEC_ON = " << spec.use_e << ", E = " << spec.e_field << " \n";
    }

    leo2d_kpm_cfg cfg{};
    cfg.poly_order = P;
    // (the complex Hamiltonian of a magnetic field runs the FP32 recursion only)
    cfg.precision = spec.precision >= 0 ? spec.precision
                                        : ((spec.observable_type == 1 || cpx_run) ? LEO2D_FP32 : LEO2D_FP64);
    cfg.block = spec.block;
    cfg.seed = spec.seed;

    if (spec.observable_type == 0 && spec.kpm_trace == 1) {
      // rootChebSolve's trace samples (locality.cpp:2254-2309)
      int S = spec.kpm_trace_samps;
      if (S == -1) {
        S = (int)1.0e6 / ((double)n);
        if (S < 1) S = 1;
        if (S > 100) S = 100;
      }
      cfg.num_vectors = S;
      std::vector<double> mu((size_t)S * P);
      if (spec.vectors == 0) {
        std::vector<double> vec((size_t)S * n_kpm);
        for (int s = 0; s < S; ++s)
          for (int64_t i = 0; i < n_kpm; ++i) vec[(size_t)s * n_kpm + i] = distribution(generator);
        cfg.vector_kind = LEO2D_VEC_HOST;
        CHECK(leo2d_kpm_dos(ctx.h, kcsr, &cfg, vec.data(), mu.data()));
      } else {
        cfg.vector_kind = LEO2D_VEC_PHASE;
        CHECK(leo2d_kpm_dos(ctx.h, kcsr, &cfg, nullptr, mu.data()));
      }
      std::vector<double> dos(P), Ek(P);
      // densityTransformTrace(results, 1/num_dofs) (locality.cpp:3126-3131); a
      // vacancy job's num_dofs takes its vacancies off the reduced size again
      const double num_dofs = (double)(n_kpm - n_vac);
      CHECK(leo2d_dos_transform(ctx.h, mu.data(), P, S, rescale, shift, 1.0 / num_dofs, dos.data(), Ek.data()));
      if (spec.mlmc == 1) {  // Mlmc_handler::process (mlmc_handler.cpp:118-178)
        const VacJob& vj = vjobs[job];
        if (vj.cluster_id == -1) {
          MlmcStats::update(mlmc.E, mlmc.nE, dos);
          MlmcStats::update(mlmc.V, mlmc.nV, MlmcStats::square(dos));
          if (spec.mlmc_level > 1 &&
              !MlmcStats::save(mlmc_name(mlmc_temp, spec.job_name, spec.mlmc_level,
                                         "_J" + std::to_string(vj.mlmc_id) + "_dos.bin"), dos)) {
            err = "cannot write the MLMC job file under " + mlmc_temp;
            return LEO2D_ERR_IO;
          }
        } else {
          if (vj.cluster_id < 1 || vj.cluster_id > (int)mlmc.cluster_original.size()) {
            err = "CLUSTERID " + std::to_string(vj.cluster_id) + " is outside MLMC_NUM_CLUSTERS";
            return LEO2D_ERR_BAD_ARG;
          }
          const std::vector<double> d = MlmcStats::diff(mlmc.cluster_original[vj.cluster_id - 1], dos);
          MlmcStats::update(mlmc.DE, mlmc.nDE, d);
          MlmcStats::update(mlmc.DV, mlmc.nDV, MlmcStats::square(d));
        }
        continue;
      }
      if (spec.verbose_save == 1) {
        if (first_job) {
          cheb << "E: ";
          write_energies(cheb, E);
        }
        cheb << "T: \n";
        // save() prints cheb_coeffs rows for the job's target list (param_tools.cpp:65-71)
        for (size_t t = 0; t < targets.size() && t < (size_t)S; ++t) {
          cheb << targets[t] << ": ";
          for (int j = 0; j < P - 1; ++j) cheb << mu[t * P + j] << ", ";
          cheb << mu[t * P + P - 1] << "\n";
        }
        cheb << "\n";
      } else {
        if (first_job) write_energies(cheb, E);
        for (int j = 0; j < P - 1; ++j) cheb << dos[j] << " ";
        cheb << dos[P - 1] << "\n";
      }
      if (spec.energies > 0) {
        std::vector<double> mean(P, 0.0), Eg(spec.energies), d(spec.energies);
        for (int s = 0; s < S; ++s)
          for (int j = 0; j < P; ++j) mean[j] += mu[(size_t)s * P + j] / S;
        for (int k = 0; k < spec.energies; ++k)
          Eg[k] = center + rescale * (-1.0 + 2.0 * (k + 0.5) / spec.energies);
        CHECK(leo2d_dos_reconstruct(ctx.h, mean.data(), P, Eg.data(), spec.energies, rescale, center,
                                    1.0 / (double)n, d.data()));
        std::ofstream f(join_path(out_dir, spec.job_name + "_dos.dat"));
        f << std::setprecision(17);
        for (int k = 0; k < spec.energies; ++k) f << Eg[k] << " " << d[k] << "\n";
      }
    } else if (spec.observable_type == 0) {
      const int64_t T = (int64_t)targets.size();
      std::vector<double> mu((size_t)T * P);
      CHECK(leo2d_kpm_ldos(ctx.h, kcsr, &cfg, targets.data(), T, mu.data()));
      std::vector<double> out = mu;
      if (spec.dos_transform == 1) {  // Param_tools::densityTransform
        std::vector<double> Ek(P);
        for (int64_t t = 0; t < T; ++t)
          CHECK(leo2d_dos_transform(ctx.h, mu.data() + t * P, P, 1, rescale, shift, 1.0, out.data() + t * P,
                                    Ek.data()));
      }
      if (spec.verbose_save == 1) {
        if (first_job) {
          cheb << "E: ";
          write_energies(cheb, E);
        }
        cheb << "T: \n";
        for (int64_t t = 0; t < T; ++t) {
          cheb << targets[t] << ": ";
          for (int j = 0; j < P - 1; ++j) cheb << out[t * P + j] << ", ";
          cheb << out[t * P + P - 1] << "\n";
        }
        cheb << "\n";
      } else {
        if (first_job) write_energies(cheb, E);
        for (int64_t t = 0; t < T; ++t) {
          for (int j = 0; j < P - 1; ++j) cheb << out[t * P + j] << " ";
          cheb << out[t * P + P - 1] << "\n";
        }
      }
    } else {
      const int64_t T = (int64_t)targets.size();
      std::vector<double> M((size_t)T * P * P);
      CHECK(leo2d_kpm_cond(ctx.h, csr.h, &cfg, targets.data(), T, M.data()));
      std::vector<double> out = M;
      if (spec.cond_transform == 1)
        for (int64_t t = 0; t < T; ++t)
          CHECK(leo2d_cond_transform(ctx.h, M.data() + t * P * P, P, out.data() + t * P * P));
      if (spec.verbose_save == 0) {  // param_tools.cpp:288-316
        if (first_job) {
          write_energies(cheb, E);
          cheb << "\n";
        }
        for (int64_t t = 0; t < T; ++t) {
          for (int i = 0; i < P; ++i) {
            for (int j = 0; j < P; ++j) cheb << out[(size_t)t * P * P + (size_t)i * P + j] << " ";
            cheb << "\n";
          }
          cheb << "\n";
        }
      }
    }
  }  // jobs
  cheb.close();
  if (spec.mlmc == 1) {  // Mlmc_handler::save (mlmc_handler.cpp:394-481)
    const int lvl = spec.mlmc_level;
    bool ok = true;
    if (spec.kpm_trace == 1) {
      ok = ok && MlmcStats::save(mlmc_name(mlmc_out, spec.job_name, lvl, "_E_dos.bin"), mlmc.E);
      ok = ok && MlmcStats::save(mlmc_name(mlmc_out, spec.job_name, lvl, "_V_dos.bin"), mlmc.V);
    }
    std::vector<double> Ef(P);
    for (int i = 0; i < P; ++i)
      Ef[i] = spec.geom.energy_shift + spec.geom.energy_rescale * std::cos((i * 1.0 + 0.5) * M_PI / P);
    ok = ok && MlmcStats::save(mlmc_name(mlmc_out, spec.job_name, lvl, "_ENERGIES.bin"), Ef);
    if (lvl < spec.mlmc_max_level && spec.kpm_trace == 1) {
      ok = ok && MlmcStats::save(mlmc_name(mlmc_out, spec.job_name, lvl, "_DE_dos.bin"), mlmc.DE);
      ok = ok && MlmcStats::save(mlmc_name(mlmc_out, spec.job_name, lvl, "_DV_dos.bin"), mlmc.DV);
    }
    if (!ok) {
      err = "cannot write the MLMC statistics under " + mlmc_out;
      return LEO2D_ERR_IO;
    }
  }
  if (!kjobs.empty()) {  // Param_tools::saveKpts (param_tools.cpp:579-602), one line per job
    std::ofstream kf(join_path(out_dir, spec.job_name + ".kpts"));
    kf << std::fixed;
    kf.precision(10);
    for (const auto& k : kjobs) {
      if (k[0] >= 0) kf << " ";
      kf << k[0] << "\t\t";
      if (k[1] >= 0) kf << " ";
      kf << k[1] << " \n";
    }
  }

  // (the matrix and position files of the last job: the reference's jobs
  // overwrite each other's, locality.cpp:4362-4365)
  if (spec.matrix_save > 0) {  // generateRealH's matrix save (locality.cpp:4366-4383)
    std::vector<int64_t> rp(n + 1);
    std::vector<int32_t> col(nnz);
    std::vector<double> val(nnz), dx, dy;
    if (spec.matrix_save > 1) {
      dx.resize(nnz);
      dy.resize(nnz);
    }
    CHECK(leo2d_csr_download(ctx.h, csr.h, rp.data(), col.data(), val.data(),
                             dx.empty() ? nullptr : dx.data(), dy.empty() ? nullptr : dy.data()));
    if (cpx_run) {  // generateCpxH's matrix save (locality.cpp:5213-5228): every entry, re and im
      std::vector<double> im(nnz, 0.0);
      if (last_complex) CHECK(leo2d_csr_download_imag(ctx.h, csr.h, im.data()));
      std::ofstream f(join_path(out_dir, spec.job_name + "_matrix.dat"));
      for (int64_t i = 0; i < n; ++i)
        for (int64_t j = rp[i]; j < rp[i + 1]; ++j)
          f << col[j] + 1 << ", " << i + 1 << ", " << val[j] << ", " << im[j] << "\n";
    }
    auto dump = [&](const std::string& suffix, const std::vector<double>& v) {
      std::ofstream f(join_path(out_dir, spec.job_name + suffix));
      for (int64_t i = 0; i < n; ++i)
        for (int64_t j = rp[i]; j < rp[i + 1]; ++j)
          if (std::fabs(v[j]) > 1e-12) f << col[j] + 1 << ", " << i + 1 << ", " << v[j] << "\n";
    };
    if (!cpx_run) dump("_matrix.dat", val);
    if (spec.matrix_save > 1) {
      dump("_dxH_matrix.dat", dx);
      dump("_dyH_matrix.dat", dy);
    }
  }
  if (spec.matrix_pos_save > 0) {  // locality.cpp:4428-4448
    std::ofstream f(join_path(out_dir, spec.job_name + "_pos.dat"));
    f << std::fixed;
    f.precision(12);
    for (int64_t i = 0; i < n; ++i)
      f << pos[3 * i] << "    " << pos[3 * i + 1] << "    " << pos[3 * i + 2] << "    " << grid4[4 * i + 3]
        << "    " << grid4[4 * i + 2] << "\n";
  }
  return LEO2D_OK;
}

}  // namespace leo2d_host

extern "C" leo2d_status leo2d_run_input(const char* in_path, const char* out_dir, int device, char* msg,
                                        size_t msg_len) {
  std::string err;
  leo2d_status st = LEO2D_OK;
  try {
    leo2d_host::JobSpec spec;
    if (!in_path || !leo2d_host::parse_input(in_path, spec, err)) {
      st = LEO2D_ERR_IO;
    } else {
      st = leo2d_host::run_job(spec, out_dir ? out_dir : ".", device, err);
    }
  } catch (const std::exception& e) {
    err = e.what();
    st = LEO2D_ERR_CUDA;
  }
  if (msg && msg_len) {
    std::strncpy(msg, err.c_str(), msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  return st;
}

extern "C" leo2d_status leo2d_parse_input(const char* in_path, leo2d_geom* geom_out, int32_t* ints_out,
                                          char* msg, size_t msg_len) {
  std::string err;
  leo2d_host::JobSpec spec;
  leo2d_status st = LEO2D_OK;
  if (!in_path || !leo2d_host::parse_input(in_path, spec, err)) {
    st = LEO2D_ERR_IO;
  } else {
    if (geom_out) *geom_out = spec.geom;
    if (ints_out) {
      const int32_t v[10] = {spec.solver_type,    spec.observable_type, spec.poly_order,
                             spec.kpm_trace,      spec.kpm_trace_samps, spec.verbose_save,
                             spec.matrix_save,    (int32_t)spec.unsupported.size(),
                             spec.target_sheets.empty() ? -1 : spec.target_sheets[0], spec.nshifts};
      for (int i = 0; i < 10; ++i) ints_out[i] = v[i];
    }
    for (const auto& u : spec.unsupported) err += "[" + u + "] ";
  }
  if (msg && msg_len) {
    std::strncpy(msg, err.c_str(), msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  return st;
}
