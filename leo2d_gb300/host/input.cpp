// input.cpp - the .in reader of the KPM path.
//
// Same token rules as app/src/main.cpp:75-911: each line is split on single
// spaces; a keyword consumes the tokens after it ("KEY = value" reads "=" and
// "value"); numbers go through atoi/atof; unknown tokens are ignored. Sheets
// take the grid bounds and radius current when their MATERIAL line is read
// (main.cpp:324-336); ANGLE is in degrees (main.cpp:345-351). Keywords that
// select reference paths this build does not implement are collected in
// JobSpec::unsupported so the driver can refuse the job instead of silently
// computing something else.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "job.h"

namespace leo2d_host {

namespace {

std::vector<std::string> split_spaces(const std::string& line) {
  std::vector<std::string> out;
  std::istringstream ss(line);
  std::string t;
  while (std::getline(ss, t, ' ')) out.push_back(t);
  return out;
}

}  // namespace

bool parse_input(const std::string& path, JobSpec& spec, std::string& err) {
  std::ifstream in(path);
  if (!in.is_open()) {
    err = "Input file '" + path + "' not found";
    return false;
  }
  leo2d_geom& g = spec.geom;
  g = leo2d_geom{};
  g.sc_search_size = 1;  // job_params.cpp:57
  g.energy_rescale = 20.0;  // job_params.cpp:116
  g.energy_shift = 0.0;
  std::vector<int> mn, mx;  // main.cpp pushes three entries per MINSIZE / MAXSIZE
  double max_R = 0.0;
  int num_sheets = 0, current_sheet = -1;
  std::vector<int> sc_groups;  // SUPERCELL_GROUPS, 0-based group of each sheet (empty: not given)
  double height = 0.0, angle = 0.0;
  std::vector<double> heights, angles;
  std::vector<int> sheet_min0, sheet_max0;
  std::vector<double> sheet_R;
  std::vector<bool> sheet_set;
  int model = LEO2D_MODEL_REF;
  bool model_key = false;
  std::string line;
  while (std::getline(in, line)) {
    const std::vector<std::string> tk = split_spaces(line);
    for (size_t p = 0; p < tk.size(); ++p) {
      const std::string& key = tk[p];
      auto next = [&]() -> std::string { return ++p < tk.size() ? tk[p] : std::string(); };
      auto value = [&]() -> std::string { next(); return next(); };  // skip "="
      if (key == "JOB_NAME") {
        spec.job_name = value();
      } else if (key == "MAXSIZE") {
        const int v = std::atoi(value().c_str());
        mx.push_back(v); mx.push_back(v); mx.push_back(v);
        max_R = (double)v;
      } else if (key == "MINSIZE") {
        const int v = std::atoi(value().c_str());
        mn.push_back(v); mn.push_back(v); mn.push_back(v);
      } else if (key == "MAX_R") {
        max_R = std::atof(value().c_str());
      } else if (key == "BOUNDARY_CONDITION") {
        g.boundary_condition = std::atoi(value().c_str());
      } else if (key == "NUM_SHEETS") {
        num_sheets = std::atoi(value().c_str());
        if (num_sheets < 1 || num_sheets > LEO2D_MAX_SHEETS) {
          err = "NUM_SHEETS must be 1.." + std::to_string(LEO2D_MAX_SHEETS);
          return false;
        }
        heights.assign(num_sheets, 0.0);
        angles.assign(num_sheets, 0.0);
        sheet_min0.assign(num_sheets, 0);
        sheet_max0.assign(num_sheets, 0);
        sheet_R.assign(num_sheets, 0.0);
        sheet_set.assign(num_sheets, false);
      } else if (key == "SUPERCELL_M_N") {  // main.cpp:267-277: also selects supercell type 1
        next();
        g.supercell_m = std::atoi(next().c_str());
        g.supercell_n = std::atoi(next().c_str());
        g.trilayer_supercell = 0;
      } else if (key == "SUPERCELL_GROUPS") {
        // main.cpp:131-155: two groups of sheet numbers, each closed by "/"
        next();
        sc_groups.assign(num_sheets, 0);
        int placed = 0;
        for (int gc = 0; gc < 2; ++gc)
          for (std::string t = next(); !t.empty() && t != "/" && placed < num_sheets; t = next(), ++placed) {
            const int sheet = std::atoi(t.c_str()) - 1;
            if (sheet >= 0 && sheet < num_sheets) sc_groups[sheet] = gc;
          }
      } else if (key == "TRILAYER_SUPERCELL") {  // main.cpp:295-303: 1 selects supercell type 3
        if (std::atoi(value().c_str()) == 1) g.trilayer_supercell = 1;
      } else if (key == "SUPERCELL_SEARCH_SIZE") {
        g.sc_search_size = std::atoi(value().c_str());
      } else if (key == "START_SHEET") {
        current_sheet = std::atoi(next().c_str()) - 1;
        if (current_sheet + 1 > num_sheets) {
          err = "Cannot take in sheet " + std::to_string(current_sheet + 1) + " if NUM_SHEETS = " +
                std::to_string(num_sheets);
          return false;
        }
      } else if (key == "END_SHEET") {
        const int s = std::atoi(next().c_str()) - 1;
        if (current_sheet == s && s >= 0) {
          heights[s] = height;
          angles[s] = angle;
          current_sheet = -1;
        }
      } else if (key == "MATERIAL") {
        const std::string mat = value();
        if (current_sheet < 0 || current_sheet >= num_sheets) {
          err = "MATERIAL outside START_SHEET/END_SHEET";
          return false;
        }
        if (mat == "Graphene") {
          // the reference model unless MODEL = SIMPLE selects the other one
        } else {
          spec.unsupported.push_back("MATERIAL = " + mat);
        }
        sheet_min0[current_sheet] = mn.empty() ? -50 : mn[0];
        sheet_max0[current_sheet] = mx.empty() ? 50 : mx[0];
        sheet_R[current_sheet] = max_R;
        sheet_set[current_sheet] = true;
      } else if (key == "HEIGHT") {
        height = std::atof(value().c_str());
      } else if (key == "ANGLE") {
        angle = (2 * M_PI * std::atof(value().c_str())) / (360.0);
      } else if (key == "NSHIFTS") {
        spec.nshifts = std::atoi(value().c_str());
      } else if (key == "ENERGY_RESCALE") {
        g.energy_rescale = std::atof(value().c_str());
      } else if (key == "ENERGY_SHIFT") {
        g.energy_shift = std::atof(value().c_str());
      } else if (key == "POLY_ORDER") {
        spec.poly_order = std::atoi(value().c_str());
      } else if (key == "SOLVER_TYPE") {
        const std::string v = value();
        if (v == "SQ") spec.solver_type = 1;
        else if (v == "LC") spec.solver_type = 2;
        else if (v == "FIXED_SHIFT") spec.solver_type = 6;
        else if (v == "MLMC_VAC") spec.solver_type = 3;
        else if (v == "VD_FILE") spec.solver_type = 4;
        else if (v == "STRAIN")
          spec.unsupported.push_back("SOLVER_TYPE = " + v);
      } else if (key == "NUM_LC_POINTS") {
        spec.num_lc_points = std::atoi(value().c_str());
      } else if (key == "LC_POINTS") {  // main.cpp:438-454: pairs of fractions
        next();
        spec.lc_points.assign(2 * (size_t)std::max(spec.num_lc_points, 0), 0.0);
        for (size_t i = 0; i < spec.lc_points.size(); ++i) spec.lc_points[i] = std::atof(next().c_str());
      } else if (key == "OBSERVABLE_TYPE") {
        const std::string v = value();
        if (v == "DOS") spec.observable_type = 0;
        else if (v == "COND") spec.observable_type = 1;
      } else if (key == "DOS_TRANSFORM") {
        spec.dos_transform = std::atoi(value().c_str());
      } else if (key == "COND_TRANSFORM") {
        spec.cond_transform = std::atoi(value().c_str());
      } else if (key == "MATRIX_SAVE") {
        spec.matrix_save = std::atoi(value().c_str());
      } else if (key == "MATRIX_POS_SAVE") {
        spec.matrix_pos_save = std::atoi(value().c_str());
      } else if (key == "VERBOSE_SAVE") {
        spec.verbose_save = std::atoi(value().c_str());
      } else if (key == "KPM_TRACE") {
        spec.kpm_trace = std::atoi(value().c_str());
      } else if (key == "KPM_TRACE_SAMPS") {
        spec.kpm_trace_samps = std::atoi(value().c_str());
      } else if (key == "NUM_SHIFT_SHEETS") {
        spec.num_shift_sheets = std::atoi(value().c_str());
      } else if (key == "SHIFT_SHEETS") {  // main.cpp:874-884
        next();
        spec.shift_sheets.assign(spec.num_shift_sheets > 0 ? spec.num_shift_sheets : 0, 0);
        for (size_t i = 0; i < spec.shift_sheets.size(); ++i)
          spec.shift_sheets[i] = std::atoi(next().c_str()) - 1;
      } else if (key == "NUM_TARGET_SHEETS") {
        spec.num_target_sheets = std::atoi(value().c_str());
      } else if (key == "TARGET_SHEETS") {
        next();
        spec.target_sheets.assign(spec.num_target_sheets > 0 ? spec.num_target_sheets : 0, 0);
        for (size_t i = 0; i < spec.target_sheets.size(); ++i)
          spec.target_sheets[i] = std::atoi(next().c_str()) - 1;
      } else if (key == "SOLVER_SPACE") {
        if (value() == "M") spec.unsupported.push_back("SOLVER_SPACE = M");
      } else if (key == "STRAIN_TYPE") {
        const std::string v = value();
        if (std::atoi(v.c_str()) != 0) spec.unsupported.push_back("STRAIN_TYPE = " + v);
      } else if (key == "USE_B_FIELD") {
        spec.use_b = std::atoi(value().c_str());
      } else if (key == "B_FIELD") {
        spec.b_field = std::atof(value().c_str());
      } else if (key == "K_SAMPLING") {  // main.cpp:175-200
        spec.k_sampling = std::atoi(value().c_str());
      } else if (key == "K_TYPE") {
        spec.k_type = std::atoi(value().c_str());
      } else if (key == "K_GRID") {
        next();
        spec.num_k1 = std::atoi(next().c_str());
        spec.num_k2 = std::atoi(next().c_str());
      } else if (key == "USE_E_FIELD") {  // main.cpp:832-842
        spec.use_e = std::atoi(value().c_str());
      } else if (key == "E_FIELD") {
        spec.e_field = std::atof(value().c_str());
      } else if (key == "MLMC") {  // main.cpp:730-775
        spec.mlmc = std::atoi(value().c_str());
      } else if (key == "MLMC_MAX_LEVEL") {
        spec.mlmc_max_level = std::atoi(value().c_str());
      } else if (key == "MLMC_LEVEL") {
        spec.mlmc_level = std::atoi(value().c_str());
      } else if (key == "MLMC_NUM_CLUSTERS") {
        spec.mlmc_num_clusters = std::atoi(value().c_str());
      } else if (key == "MLMC_CLUSTER_SIZE") {
        spec.mlmc_cluster_size = std::atoi(value().c_str());
      } else if (key == "MLMC_OUT_ROOT") {
        spec.mlmc_out_root = value();
      } else if (key == "MLMC_TEMP_ROOT") {
        spec.mlmc_temp_root = value();
      } else if (key == "VACANCY_FILE") {
        spec.vacancy_file = value();
      } else if (key == "DIAGONALIZE" || key == "CHIRAL_ON" || key == "BALLISTIC_TRANSPORT" ||
                 key == "MAT_FROM_FILE" || key == "GLOBAL_SHIFTS_ON" || key == "UNIFORM_STRAIN" ||
                 key == "COND_POLY_PAR" || key == "MAT_SOC_ON") {
        const std::string v = value();
        if (std::atoi(v.c_str()) != 0) spec.unsupported.push_back(key + " = " + v);
      } else if (key == "MODEL") {
        const std::string v = value();
        model_key = true;
        if (v == "SIMPLE") model = LEO2D_MODEL_SIMPLE;
        else if (v == "REF") model = LEO2D_MODEL_REF;
        else spec.unsupported.push_back("MODEL = " + v);
      } else if (key == "KPM_VECTORS") {
        const std::string v = value();
        if (v == "PHASE") spec.vectors = 1;
        else if (v == "GAUSSIAN") spec.vectors = 0;
        else spec.unsupported.push_back("KPM_VECTORS = " + v);
      } else if (key == "KPM_SEED") {
        spec.seed = std::strtoull(value().c_str(), nullptr, 10);
      } else if (key == "KPM_PRECISION") {
        const std::string v = value();
        spec.precision = v == "FP32" ? LEO2D_FP32 : LEO2D_FP64;
      } else if (key == "KPM_BOUNDS") {
        spec.bounds = value() == "GERSHGORIN" ? 1 : 0;
      } else if (key == "KPM_ENERGIES") {
        spec.energies = std::atoi(value().c_str());
      } else if (key == "KPM_BLOCK") {
        spec.block = std::atoi(value().c_str());
      }
    }
  }
  g.num_sheets = num_sheets;
  g.model = model;
  (void)model_key;
  for (int s = 0; s < num_sheets; ++s) {
    if (!sheet_set[s]) {
      err = "sheet " + std::to_string(s + 1) + " has no MATERIAL";
      return false;
    }
    g.min_shape[s][0] = g.min_shape[s][1] = sheet_min0[s];
    g.max_shape[s][0] = g.max_shape[s][1] = sheet_max0[s];
    g.max_R[s] = sheet_R[s];
    g.heights[s] = heights[s];
    g.angles[s] = angles[s];
  }
  if (spec.target_sheets.empty()) spec.target_sheets.push_back(0);
  // a magnetic field: the complex Hamiltonian of generateCpxH (locality.cpp:2906-2909)
  if (spec.use_e == 1) g.e_field = spec.e_field;
  if (g.boundary_condition == 1 && g.trilayer_supercell && num_sheets != 3)
    spec.unsupported.push_back("TRILAYER_SUPERCELL = 1 with NUM_SHEETS = " + std::to_string(num_sheets));
  if (g.boundary_condition == 1 && !g.trilayer_supercell && num_sheets >= 3 && !sc_groups.empty()) {
    // the (M, N) cell here puts sheet 1 in group 1 and the others in group 2
    // (setupSupercell reads the groups for three or more sheets, locality.cpp:161-170)
    bool dflt = sc_groups[0] == 0;
    for (int s = 1; s < num_sheets; ++s) dflt = dflt && sc_groups[s] == 1;
    if (!dflt) spec.unsupported.push_back("SUPERCELL_GROUPS other than 1 / 2 .. NUM_SHEETS /");
  }
  if (spec.k_sampling == 1) {
    if (spec.k_type < 0 || spec.k_type > 5) spec.unsupported.push_back("K_TYPE = " + std::to_string(spec.k_type));
    if (g.boundary_condition != 1) spec.unsupported.push_back("K_SAMPLING = 1 with BOUNDARY_CONDITION = 0");
    if (spec.observable_type == 1) spec.unsupported.push_back("K_SAMPLING = 1 with OBSERVABLE_TYPE = COND");
  }
  if (spec.use_b == 1) {
    g.b_field = spec.b_field;
    if (spec.observable_type == 1) spec.unsupported.push_back("USE_B_FIELD = 1 with OBSERVABLE_TYPE = COND");
  }
  return true;
}

}  // namespace leo2d_host
