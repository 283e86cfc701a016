// job.h - host-side description of a LEO2D KPM job (what app/src/main.cpp
// collects into Sdata and Job_params for this path) and the driver around the
// C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/leo2d_gpu.h"

namespace leo2d_host {

// Parsed input: the .in keywords the KPM path reads (main.cpp:75-911) with
// the reference's defaults (job_params.cpp:17-225), plus the additive keys of
// this implementation (MODEL, KPM_VECTORS, KPM_SEED, KPM_PRECISION,
// KPM_BOUNDS, KPM_ENERGIES, KPM_BLOCK).
struct JobSpec {
  std::string job_name = "LEO2D_JOB";
  leo2d_geom geom{};
  int solver_type = 0;        // SOLVER_TYPE: 1 = SQ, 2 = LC, 3 = MLMC_VAC, 4 = VD_FILE, 6 = FIXED_SHIFT
  int num_lc_points = 0;      // NUM_LC_POINTS (LC: the polyline of shifts of the last sheet)
  std::vector<double> lc_points;  // LC_POINTS, (s1, s2) pairs
  int observable_type = 0;    // 0 = DOS, 1 = COND
  int poly_order = 20;
  int kpm_trace = 0;
  int kpm_trace_samps = -1;
  int dos_transform = 1;
  int cond_transform = 1;
  int matrix_save = 0;
  int matrix_pos_save = 0;
  int verbose_save = 1;
  int nshifts = 1;            // NSHIFTS: an N x N grid of shifts per shift sheet
  int num_shift_sheets = 1;   // NUM_SHIFT_SHEETS (job_params.cpp:44)
  std::vector<int> shift_sheets;  // SHIFT_SHEETS, 0-based
  int num_target_sheets = 1;
  std::vector<int> target_sheets;  // 0-based
  // additive keys
  int vectors = 0;            // 0 = reference Gaussian (std::normal_distribution), 1 = random phase
  uint64_t seed = 0;
  int precision = -1;         // -1: the path's default (DOS FP64 as the reference, Kubo FP32)
  int bounds = 0;             // 0 = ENERGY_RESCALE/SHIFT as given, 1 = Gershgorin x 1.01
  int use_b = 0;              // USE_B_FIELD: the complex Hamiltonian (generateCpxH)
  double b_field = 0.0;       // B_FIELD, tesla
  int use_e = 0;              // USE_E_FIELD: the on-site z E term
  int k_sampling = 0;         // K_SAMPLING: every job at each point of a k grid (complex H)
  int k_type = 0;             // K_TYPE (0 = grid of the supercell's Brillouin zone; 1-4 zone paths)
  int num_k1 = 1, num_k2 = 1; // K_GRID
  double e_field = 0.0;       // E_FIELD
  int energies = 0;           // > 0: also write a DOS on this many equispaced energies
  // multilevel Monte Carlo over vacancy configurations (job_params.cpp:131-152)
  int mlmc = 0;               // MLMC: 1 = the jobs' results go to the level statistics, no .cheb
  int mlmc_level = 0;         // MLMC_LEVEL
  int mlmc_max_level = 1;     // MLMC_MAX_LEVEL
  int mlmc_num_clusters = 0;  // MLMC_NUM_CLUSTERS
  int mlmc_cluster_size = 4;  // MLMC_CLUSTER_SIZE
  std::string mlmc_out_root = "out";    // MLMC_OUT_ROOT
  std::string mlmc_temp_root = "temp";  // MLMC_TEMP_ROOT
  std::string vacancy_file = "vacancies.dat";  // VACANCY_FILE (MLMC_VAC jobs)
  int block = 0;
  std::vector<std::string> unsupported;  // keys that select paths outside this build
};

// Parses a .in file with main.cpp's token rules. Returns false if unreadable.
bool parse_input(const std::string& path, JobSpec& spec, std::string& err);

// Runs the job through the C ABI on `device` and writes <job>.cheb (and
// <job>_matrix.dat / <job>_pos.dat when asked) into `out_dir`.
leo2d_status run_job(const JobSpec& spec, const std::string& out_dir, int device, std::string& err);

}  // namespace leo2d_host
