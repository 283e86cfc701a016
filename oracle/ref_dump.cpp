/*
 * ref_dump: drives the reference's own KPM-path functions on one job and
 * writes their internal arrays to binary files.
 *
 * TEST INFRASTRUCTURE ONLY. Built by oracle/Makefile.ref from the reference
 * sources where they lie (never copied) into oracle/_ref/. It is used here, in
 * the build container, to generate the golden fixtures under tests/golden/;
 * nothing on the GPU path runs it.
 *
 * It repeats the rank-0 half of Locality::constructGeom
 * (src/locality.cpp:822-1060: Sheet, Hstruct, getInterPairs, getIntraPairs,
 * getIndexToPos) and the worker half of workerChebSolve for job 1 with zero
 * shifts (src/locality.cpp:2935-3148: setConfigPositions, generateRealH,
 * computeDosKPM / computeDosTraceKPM / computeCondKPM), calling the
 * reference's methods. Trace vectors are drawn exactly as rootChebSolve does
 * (src/locality.cpp:2254-2309): one default-constructed
 * std::default_random_engine and std::normal_distribution<double>(0,1).
 *
 * Input: a LEO2D .in file (the subset of keywords main.cpp:75-911 uses for a
 * real-space graphene KPM job). Output directory: argv[2].
 */
#include <pthread.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#define private public
#define protected public
#include "locality.h"
#include "params/param_tools.h"
#undef private
#undef protected

namespace {

template <class T>
void dump(const std::string& dir, const std::string& name, const T* p, size_t n) {
  std::string path = dir + "/" + name + ".bin";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  if (n) std::fwrite(p, sizeof(T), n, f);
  std::fclose(f);
}

std::vector<std::string> tokens(const std::string& line) {
  std::vector<std::string> out;
  std::istringstream ss(line);
  std::string t;
  while (std::getline(ss, t, ' ')) out.push_back(t);
  return out;
}

}  // namespace

static int dump_main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_dump file.in outdir\n");
    return 2;
  }
  const std::string outdir = argv[2];

  // ---- .in subset, same token rules as app/src/main.cpp:75-911 ----
  int min_size = -50, max_size = 50, boundary_condition = 0;
  std::vector<int> mn, mx;
  double max_R = 0;
  int num_sheets = 0, current_sheet = -1;
  std::vector<Sdata> s_data;
  std::vector<double> heights, angles;
  double height = 0, angle = 0;
  std::string strain_file;
  Job_params opts;
  // (this driver only) orbitals removed from the matrix, 0-based, as the
  // vacancy solvers hand generateRealH a job's vacancy_list
  std::vector<int> vacancies;
  // (this driver only) a Bloch vector (1/A): the job of a k-sampled run with that k_vec
  std::vector<double> k_vec;
  // (this driver only) a sheet shift "sheet,s1,s2" (1-based sheet, fractions of
  // its lattice vectors): the job of a shifted configuration
  std::vector<double> dump_shift;

  std::ifstream in(argv[1]);
  if (!in.is_open()) { std::fprintf(stderr, "cannot open %s\n", argv[1]); return 2; }
  std::string line;
  while (std::getline(in, line)) {
    std::vector<std::string> tk = tokens(line);
    for (size_t p = 0; p < tk.size(); ++p) {
      const std::string& key = tk[p];
      auto val = [&](size_t k) { return p + k < tk.size() ? tk[p + k] : std::string(); };
      if (key == "JOB_NAME") opts.setParam("job_name", val(2));
      if (key == "REF_DUMP_SHIFT") {
        std::istringstream ss(val(2));
        std::string t;
        while (std::getline(ss, t, ',')) dump_shift.push_back(std::atof(t.c_str()));
      }
      if (key == "REF_DUMP_KVEC") {
        std::istringstream ks(val(2));
        std::string t;
        while (std::getline(ks, t, ',')) k_vec.push_back(std::atof(t.c_str()));
      }
      if (key == "REF_DUMP_VACANCIES") {
        std::istringstream vs(val(2));
        std::string t;
        while (std::getline(vs, t, ',')) vacancies.push_back(std::atoi(t.c_str()));
      }
      if (key == "MAXSIZE") {
        max_size = std::atoi(val(2).c_str());
        mx.push_back(max_size); mx.push_back(max_size); mx.push_back(max_size);
        max_R = (double)max_size;
      }
      if (key == "MINSIZE") {
        min_size = std::atoi(val(2).c_str());
        mn.push_back(min_size); mn.push_back(min_size); mn.push_back(min_size);
      }
      if (key == "MAX_R") max_R = std::atof(val(2).c_str());
      if (key == "BOUNDARY_CONDITION") {
        boundary_condition = std::atoi(val(2).c_str());
        opts.setParam("boundary_condition", boundary_condition);
      }
      if (key == "NUM_SHEETS") {
        num_sheets = std::atoi(val(2).c_str());
        s_data.resize(num_sheets); heights.resize(num_sheets); angles.resize(num_sheets);
        opts.setParam("num_sheets", num_sheets);
      }
      if (key == "SUPERCELL_M_N") {
        opts.setParam("m_supercell", std::atoi(val(2).c_str()));
        opts.setParam("n_supercell", std::atoi(val(3).c_str()));
        int one = 1;
        opts.setParam("supercell_type", one);
      }
      if (key == "TRILAYER_SUPERCELL" && std::atoi(val(2).c_str()) == 1) {  // main.cpp:295-303
        int three = 3;
        opts.setParam("supercell_type", three);
      }
      if (key == "START_SHEET") current_sheet = std::atoi(val(1).c_str()) - 1;
      if (key == "END_SHEET") {
        if (current_sheet == std::atoi(val(1).c_str()) - 1) {
          heights[current_sheet] = height;
          angles[current_sheet] = angle;
          current_sheet = -1;
        }
      }
      if (key == "MATERIAL") {
        Materials::Mat mat = Materials::string_to_mat(val(2));
        s_data[current_sheet] = Sdata(mat, mn, mx, max_R, boundary_condition, 0, 0, strain_file, 0);
      }
      if (key == "HEIGHT") height = std::atof(val(2).c_str());
      if (key == "ANGLE") angle = (2 * M_PI * std::atof(val(2).c_str())) / (360.0);
      if (key == "ENERGY_RESCALE") opts.setParam("energy_rescale", std::atof(val(2).c_str()));
      if (key == "ENERGY_SHIFT") opts.setParam("energy_shift", std::atof(val(2).c_str()));
      if (key == "POLY_ORDER") opts.setParam("poly_order", std::atoi(val(2).c_str()));
      if (key == "USE_B_FIELD") opts.setParam("magOn", std::atoi(val(2).c_str()));
      if (key == "B_FIELD") opts.setParam("B", std::atof(val(2).c_str()));
      if (key == "USE_E_FIELD") opts.setParam("elecOn", std::atoi(val(2).c_str()));
      if (key == "E_FIELD") opts.setParam("E", std::atof(val(2).c_str()));
      if (key == "SOLVER_TYPE" && val(2) == "SQ") opts.setParam("solver_type", 1);
      if (key == "SOLVER_TYPE" && val(2) == "LC") opts.setParam("solver_type", 2);
      if (key == "SOLVER_TYPE" && val(2) == "FIXED_SHIFT") opts.setParam("solver_type", 6);
      if (key == "OBSERVABLE_TYPE") {
        if (val(2) == "DOS") opts.setParam("observable_type", 0);
        if (val(2) == "COND") opts.setParam("observable_type", 1);
      }
      if (key == "KPM_TRACE") opts.setParam("kpm_trace", std::atoi(val(2).c_str()));
      if (key == "KPM_TRACE_SAMPS") opts.setParam("kpm_trace_samps", std::atoi(val(2).c_str()));
      if (key == "NUM_TARGET_SHEETS") opts.setParam("num_target_sheets", std::atoi(val(2).c_str()));
      if (key == "TARGET_SHEETS") {
        std::vector<int> ts(opts.getInt("num_target_sheets"));
        for (size_t i = 0; i < ts.size(); ++i) ts[i] = std::atoi(val(2 + i).c_str()) - 1;
        opts.setParam("target_sheets", ts);
      }
    }
  }
  for (int i = 0; i < num_sheets; ++i) {
    s_data[i].solver_space = opts.getInt("solver_space");
    s_data[i].strain_type = opts.getInt("strain_type");
    s_data[i].sheet_index = i;
    s_data[i].opts = opts;
  }

  // ---- Locality set-up (rank 0 of 2, no MPI traffic is made below) ----
  Locality loc(s_data, heights, angles);
  loc.rank = 0;
  loc.size = 2;
  loc.root = 0;
  loc.print_rank = 1;
  loc.setup(opts);
  Job_params& O = loc.opts;

  // ---- rank-0 geometry, as constructGeom does ----
  std::vector<Sheet> sheets;
  for (size_t i = 0; i < loc.sdata.size(); ++i) sheets.push_back(Sheet(loc.sdata[i]));
  Hstruct h(sheets, loc.angles, loc.heights, O.getInt("solver_space"), O);
  const int N = h.getMaxIndex();
  loc.max_index = N;
  std::vector<std::vector<int>> targets = h.getTargetList(O);

  std::vector<std::vector<int>> index_vec = h.getIndexArray();
  std::vector<int> index_to_grid(4 * (size_t)N);
  for (int k = 0; k < N; ++k)
    for (int d = 0; d < 4; ++d) index_to_grid[4 * (size_t)k + d] = index_vec[k][d];

  // per-orbital local disregistry (Hstruct::getShiftConfigs, hstruct.cpp:672-820; bilayers only)
  std::vector<double> disregistry;
  if (loc.sdata.size() == 2) {
    std::vector<std::vector<double>> cfg_arr;
    h.getShiftConfigs(cfg_arr, O);
    disregistry.resize(2 * (size_t)N);
    for (int k = 0; k < N; ++k) {
      disregistry[2 * (size_t)k] = cfg_arr[k][0];
      disregistry[2 * (size_t)k + 1] = cfg_arr[k][1];
    }
  }

  std::vector<std::vector<int>> inter_vec, inter_sc;
  h.getInterPairs(inter_vec, inter_sc, O);
  std::vector<int> intra_i, intra_j;
  std::vector<double> intra_t;
  std::vector<std::vector<int>> intra_sc;
  h.getIntraPairs(intra_i, intra_j, intra_t, intra_sc, O);
  loc.max_inter_pairs = (int)inter_vec.size();
  loc.max_intra_pairs = (int)intra_i.size();

  std::vector<int> inter_pairs(2 * inter_vec.size()), intra_pairs(2 * intra_i.size());
  std::vector<int> inter_scf(2 * inter_vec.size(), 0), intra_scf(2 * intra_i.size(), 0);
  for (size_t x = 0; x < inter_vec.size(); ++x) {
    inter_pairs[2 * x] = inter_vec[x][0];
    inter_pairs[2 * x + 1] = inter_vec[x][1];
    inter_scf[2 * x] = inter_sc[x][0];
    inter_scf[2 * x + 1] = inter_sc[x][1];
  }
  for (size_t x = 0; x < intra_i.size(); ++x) {
    intra_pairs[2 * x] = intra_i[x];
    intra_pairs[2 * x + 1] = intra_j[x];
    intra_scf[2 * x] = intra_sc[x][0];
    intra_scf[2 * x + 1] = intra_sc[x][1];
  }
  std::vector<double> index_to_pos(3 * (size_t)N);
  {
    std::vector<double> px(N), py(N), pz(N);
    h.getIndexToPos(px.data(), 0);
    h.getIndexToPos(py.data(), 1);
    h.getIndexToPos(pz.data(), 2);
    for (int k = 0; k < N; ++k) {
      index_to_pos[3 * (size_t)k] = px[k];
      index_to_pos[3 * (size_t)k + 1] = py[k];
      index_to_pos[3 * (size_t)k + 2] = pz[k];
    }
  }

  // ---- job 1, shifts = 0, as rootChebSolve + workerChebSolve build it ----
  const int num_s = (int)loc.sdata.size();
  std::vector<std::vector<double>> shifts(num_s, std::vector<double>(3, 0.0));
  // the fixed-shift solver's one job (locality.cpp:1580-1608)
  if (O.getInt("solver_type") == 6)
    for (int s = 1; s < num_s; ++s) shifts[s][0] = shifts[s][1] = 1.0 / 3.0;
  if (dump_shift.size() == 3) {
    shifts[(int)dump_shift[0] - 1][0] = dump_shift[1];
    shifts[(int)dump_shift[0] - 1][1] = dump_shift[2];
  }
  // a vacancy list takes the MLMC_VAC solver's path through generateRealH and
  // the KPM functions (solver_type 3, locality.cpp:1392-1450, 2985-3016)
  if (!vacancies.empty()) O.setParam("solver_type", 3);
  // a k vector takes the k-sampling path: the worker builds the complex H
  // (locality.cpp:2906-2909) with the job's k_vec (generateCpxH, 4517-4524)
  if (k_vec.size() == 2) O.setParam("k_sampling", 1);
  Job_params job(O);
  if (k_vec.size() == 2) job.setParam("k_vec", k_vec);
  if (!vacancies.empty()) {
    job.setParam("num_vacancies", (int)vacancies.size());
    job.setParam("vacancy_list", vacancies);
  }
  // the relabelling of workerChebSolve (locality.cpp:2989-3016): reduction[i] =
  // vacancies below orbital i; the matrix keeps max_index - vacancies rows
  std::vector<int> cir(N + 1, 0);
  int Nloc = N;
  if (!vacancies.empty()) {
    int counter = 0;
    for (int i = 0; i < N; ++i) {
      cir[i] = counter;
      for (int v : vacancies)
        if (v == i) {
          ++counter;
          break;
        }
    }
    cir[N] = counter;
    Nloc = N - counter;
  }
  job.setParam("shifts", shifts);
  job.setParam("jobID", 1);
  job.setParam("max_jobs", 1);
  std::vector<int> tl = targets.empty() ? std::vector<int>() : targets[0];
  job.setParam("num_targets", (int)tl.size());
  job.setParam("target_list", tl);

  const int kpm_trace = O.getInt("kpm_trace");
  std::vector<std::vector<double>> trace_vectors;
  if (kpm_trace == 1) {
    int S = O.getInt("kpm_trace_samps");
    if (S == -1) {
      S = (int)1.0e6 / ((double)N);
      if (S < 1) S = 1;
      if (S > 100) S = 100;
    }
    std::default_random_engine generator;
    std::normal_distribution<double> distribution(0.0, 1.0);
    // (rootChebSolve draws vectors of the reduced length, locality.cpp:2280-2300)
    trace_vectors.assign(S, std::vector<double>(Nloc));
    for (int s = 0; s < S; ++s)
      for (int i = 0; i < Nloc; ++i) trace_vectors[s][i] = distribution(generator);
    job.setParam("kpm_trace_vectors", trace_vectors);
    job.setParam("num_targets", S);
  }

  std::vector<double> i2pos(3 * (size_t)N);
  std::vector<std::vector<double>> s_configs, shift_configs;
  std::vector<std::vector<std::vector<double>>> strain;
  loc.setConfigPositions(i2pos.data(), index_to_pos.data(), index_to_grid.data(), s_configs,
                         shift_configs, strain, job);

  const int num_targets = job.getInt("num_targets");
  SpMatrix H, dxH, dyH;
  std::vector<double> a0x((size_t)num_targets * Nloc + 1), a0y((size_t)num_targets * Nloc + 1);
  // a magnetic field makes the worker build the complex Hamiltonian
  // (locality.cpp:2906-2909, 3061-3071): generateCpxH with no SOC terms
  const bool cpx = O.getInt("magOn") == 1 || O.getInt("k_sampling") == 1;
  if (cpx) {
    SpMatrix jbx, jby, jtx, jty, jtbx, jtby;
    std::vector<std::vector<int>> soc_pairs;
    std::vector<std::complex<double>> soc_terms;
    loc.generateCpxH(H, dxH, dyH, jbx, jby, jtx, jty, jtbx, jtby, a0x.data(), a0y.data(), job,
                     index_to_grid.data(), i2pos.data(), inter_pairs.data(), inter_sc, intra_pairs.data(),
                     intra_t.data(), soc_pairs, soc_terms, intra_sc, strain, cir, Nloc);
  } else {
    loc.generateRealH(H, dxH, dyH, a0x.data(), a0y.data(), job, index_to_grid.data(), i2pos.data(),
                      inter_pairs.data(), inter_sc, intra_pairs.data(), intra_t.data(), intra_sc,
                      strain, cir, Nloc);
  }

  const int nnz = H.rowPointer[Nloc];
  int meta[8] = {N, nnz, loc.max_intra_pairs, loc.max_inter_pairs, num_targets,
                 O.getInt("poly_order"), kpm_trace, O.getInt("observable_type")};
  if (!vacancies.empty()) {
    // the matrix has Nloc rows; meta keeps the full orbital count
    dump(outdir, "vacancies", vacancies.data(), vacancies.size());
    int nl = Nloc;
    dump(outdir, "n_kept", &nl, 1);
  }
  dump(outdir, "meta", meta, 8);
  dump(outdir, "index_to_grid", index_to_grid.data(), index_to_grid.size());
  dump(outdir, "index_to_pos", index_to_pos.data(), index_to_pos.size());
  dump(outdir, "i2pos", i2pos.data(), i2pos.size());
  dump(outdir, "intra_pairs", intra_pairs.data(), intra_pairs.size());
  dump(outdir, "intra_t", intra_t.data(), intra_t.size());
  dump(outdir, "intra_sc", intra_scf.data(), intra_scf.size());
  dump(outdir, "inter_pairs", inter_pairs.data(), inter_pairs.size());
  dump(outdir, "inter_sc", inter_scf.data(), inter_scf.size());
  dump(outdir, "rowptr", H.rowPointer, (size_t)Nloc + 1);
  dump(outdir, "col", H.colIndex, (size_t)nnz);
  if (cpx) {
    std::vector<double> re((size_t)nnz), im((size_t)nnz);
    for (int e = 0; e < nnz; ++e) {
      re[e] = H.val_c[e].real();
      im[e] = H.val_c[e].imag();
    }
    dump(outdir, "val", re.data(), re.size());
    dump(outdir, "val_im", im.data(), im.size());
  } else {
    dump(outdir, "val", H.val, (size_t)nnz);
    dump(outdir, "val_dx", dxH.val, (size_t)nnz);
    dump(outdir, "val_dy", dyH.val, (size_t)nnz);
  }
  dump(outdir, "targets", tl.data(), tl.size());
  if (!disregistry.empty()) dump(outdir, "shift_configs", disregistry.data(), disregistry.size());

  const int P = O.getInt("poly_order");
  const int observable = O.getInt("observable_type");
  if (observable == 0) {
    std::vector<std::vector<double>> cheb(num_targets, std::vector<double>(P));
    if (kpm_trace == 0) loc.computeDosKPM(cheb, H, job, cir, Nloc);
    else loc.computeDosTraceKPM(cheb, H, job, cir, Nloc);
    std::vector<double> flat;
    for (auto& r : cheb) flat.insert(flat.end(), r.begin(), r.end());
    dump(outdir, "moments", flat.data(), flat.size());
    if (kpm_trace == 1) {
      std::vector<double> tv;
      for (auto& r : trace_vectors) tv.insert(tv.end(), r.begin(), r.end());
      dump(outdir, "trace_vectors", tv.data(), tv.size());
      Job_params res(job);
      res.setParam("cheb_coeffs", cheb);
      // the worker's DOS scale, 1 / (local_max_index - num_vacancies)
      // (locality.cpp:3124-3128): the vacancies are subtracted a second time
      Param_tools::densityTransformTrace(res, 1.0 / (double)(Nloc - (int)vacancies.size()));
      std::vector<double> dos = res.getDoubleVec("kpm_trace_dos");
      dump(outdir, "dos", dos.data(), dos.size());
    } else {
      Job_params res(job);
      res.setParam("cheb_coeffs", cheb);
      Param_tools::densityTransform(res);
      std::vector<std::vector<double>> d = res.getDoubleMat("cheb_coeffs");
      std::vector<double> df;
      for (auto& r : d) df.insert(df.end(), r.begin(), r.end());
      dump(outdir, "dos", df.data(), df.size());
    }
  } else {
    std::vector<std::vector<double>> cheb(num_targets, std::vector<double>((size_t)P * P));
    loc.computeCondKPM(cheb, H, dxH, job, cir, Nloc, a0x.data());
    std::vector<double> flat;
    for (auto& r : cheb) flat.insert(flat.end(), r.begin(), r.end());
    dump(outdir, "cond_moments", flat.data(), flat.size());
    dump(outdir, "alpha0_x", a0x.data(), (size_t)num_targets * Nloc);
    Job_params res(job);
    res.setParam("kpm_M_xx", cheb);
    Param_tools::conductivityTransform(res);
    std::vector<std::vector<double>> d = res.getDoubleMat("kpm_M_xx");
    std::vector<double> df;
    for (auto& r : d) df.insert(df.end(), r.begin(), r.end());
    dump(outdir, "cond_transform", df.data(), df.size());
  }
  std::printf("ref_dump: N=%d nnz=%d intra=%d inter=%d targets=%d\n", N, nnz,
              loc.max_intra_pairs, loc.max_inter_pairs, num_targets);
  return 0;
}

// The reference keeps Chebyshev vectors and positions in stack arrays
// (src/locality.cpp:2939, 5965-5982), so the work runs on a 1 GiB stack.
namespace {
struct MainArgs {
  int argc;
  char** argv;
  int rc;
};
void* run_dump(void* p) {
  MainArgs* a = static_cast<MainArgs*>(p);
  a->rc = dump_main(a->argc, a->argv);
  return nullptr;
}
}  // namespace

int main(int argc, char** argv) {
  MainArgs a{argc, argv, 0};
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, (size_t)1 << 30);
  pthread_t th;
  if (pthread_create(&th, &attr, run_dump, &a) != 0) return 3;
  pthread_join(th, nullptr);
  return a.rc;
}
