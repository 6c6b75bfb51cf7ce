// C API of the GB300 transport library: the subset of OpenMC's
// include/openmc/capi.h that drives a fixed-source event-based run, with the
// same names, argument meanings, return codes and exported globals, so that
// openmc.lib-style ctypes bindings work unchanged.
#include <algorithm>
#include <charconv>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "h5lite.h"
#include "host_model.h"
#include "transport.h"

// ------------------------------------------------ exported error globals
// src/error.cpp:20-30, include/openmc/capi.h:279-292
extern "C" {
int OPENMC_E_UNASSIGNED = -1;
int OPENMC_E_ALLOCATE = -2;
int OPENMC_E_OUT_OF_BOUNDS = -3;
int OPENMC_E_INVALID_SIZE = -4;
int OPENMC_E_INVALID_ARGUMENT = -5;
int OPENMC_E_INVALID_TYPE = -6;
int OPENMC_E_INVALID_ID = -7;
int OPENMC_E_GEOMETRY = -8;
int OPENMC_E_DATA = -9;
int OPENMC_E_PHYSICS = -10;
int OPENMC_E_WARNING = 1;
char openmc_err_msg[256] = {0};

// exported settings / simulation globals read through ctypes in_dll
// (include/openmc/settings.h:67-132, include/openmc/simulation.h:26-38)
bool event_based = false;
int64_t n_particles = 0;
int32_t n_inactive = 0;
int32_t gen_per_batch = 1;
int32_t max_lost_particles = 10;
double rel_max_lost_particles = 1.0e-6;
bool run_CE = true;
int verbosity = 7;
bool weight_windows_on = false;
bool restart_run = false;
bool cmfd_run = false;
bool entropy_on = false;
bool output_summary = false;
bool photon_transport = false;
bool reduce_tallies = true;
bool trigger_on = false;
bool need_depletion_rx = false;
int run_mode = 1;  // fixed source
const char* path_statepoint_c = "";
int current_batch = 0;
int current_gen = 0;
int32_t n_realizations = 0;  // active batches realised (simulation::n_realizations)
bool initialized = false;
int n_lost_particles = 0;
double keff = 1.0;
double keff_std = 0.0;
int n_coord_levels = 0;
bool DAGMC_ENABLED = false;
bool LIBMESH_ENABLED = false;
bool UWUW_ENABLED = false;
// GB300 extensions (no counterpart in the reference)
int openmc_gb300_profile_next = 0;      // 1: run the next batch kernel by kernel with event timing,
                                        // 2: every batch (graph-free, for kernel profilers)
int openmc_gb300_fuse = 3;              // bit 0: cross-section event, bit 1: surface crossing, inside the advance kernel
int64_t openmc_gb300_tail_threshold = -1;  // queue length that starts the history-based tail (-1: default)
int64_t openmc_gb300_secondary_capacity = 0;  // secondary-site pool entries (0: automatic)
int openmc_gb300_split_to_slots = 0;  // split particles start in free slots with their own seeds
int openmc_gb300_stage_tables = 0;    // event kernels copy the geometry/material tables into shared memory
int openmc_gb300_max_levels = 0;      // coordinate depth of the transport kernels (0: from the model)
int openmc_gb300_xs_fp32 = -1;          // -1: from XML (<gb300_xs_precision>), else 0/1
int openmc_gb300_contract = 1;          // FP32-table mode: transport build with fused FP64 multiply-adds
int openmc_gb300_defer_tally = 1;       // track-length tallies scored by their own kernel from track records
int64_t openmc_gb300_in_flight = 0;     // particle slots; 0: setting or automatic
int openmc_gb300_sort = 1;              // sort the XS queue by (material, energy)
int openmc_gb300_trace_batch = 1;       // batch whose histories openmc_gb300_set_trace records
int64_t openmc_gb300_trace_first = 1;   // first particle id openmc_gb300_set_trace records
}

namespace {

using namespace omc;

extern "C" int openmc_get_keff(double k_combined[]);

struct State {
  bool model_loaded = false;
  HModel model;
  GpuSim* gpu = nullptr;
  int64_t seed = 1;
  uint64_t stride = 152917ULL;
  std::vector<double> global_tallies;  // [4][3] K_COL, K_ABS, K_TRACK, LEAKAGE x (VAL, SUM, SUM_SQ)
  double time_active = 0.0;            // seconds of active-batch transport (device events)
  double time_inactive = 0.0;
  double time_wall_active = 0.0;
  int n_batches_run = 0;
  BatchStats last;
  long long trace_hist = 0;
  int trace_cap = 0;
  bool ww_user_set = false;
  // eigenvalue run (src/eigenvalue.cpp): every generation's track-length k,
  // the running sums of the active ones, and the cross sums of the three
  // estimators for the combined k
  std::vector<double> k_generation;
  double k_sum[2] = {0.0, 0.0};
  double k_col_abs = 0.0, k_col_tra = 0.0, k_abs_tra = 0.0;
  long long fission_sites = 0;
};

State& S()
{
  static State s;
  return s;
}

void set_errmsg(const std::string& m)
{
  std::snprintf(openmc_err_msg, sizeof(openmc_err_msg), "%s", m.c_str());
}

int fail(int code, const std::string& m)
{
  set_errmsg(m);
  return code;
}

void sync_globals_from_model()
{
  HModel& m = S().model;
  n_particles = m.n_particles;
  n_inactive = m.n_inactive;
  weight_windows_on = m.ww_on;
  n_coord_levels = m.n_coord_levels;
  max_lost_particles = m.max_lost_particles;
  rel_max_lost_particles = m.rel_max_lost_particles;
  event_based = m.event_based;
}

// WeightWindowsGenerator construction + create_tally
// (src/weight_windows.cpp:834-962): a WeightWindows object with invalid
// bounds and a flux tally over [mesh, energy, particle].
void setup_generators(HModel& m)
{
  for (auto& g : m.ww_generators) {
    if (g.ww >= 0) continue;
    HWeightWindows w;
    w.id = static_cast<int>(m.weight_windows.size()) + 1;
    w.mesh = g.mesh;
    w.ebounds = g.ebounds.empty() ? std::vector<double> {m.energy_min, m.energy_max} : g.ebounds;
    size_t n = (w.ebounds.size() - 1) * static_cast<size_t>(m.meshes[g.mesh].n_bins());
    w.lower.assign(n, -1.0);
    w.upper.assign(n, -1.0);
    g.ww = static_cast<int>(m.weight_windows.size());
    m.weight_windows.push_back(std::move(w));
    int fid = 1;
    for (const auto& f : m.filters) fid = std::max(fid, f.id + 1);
    int mesh_filter = -1;
    for (size_t k = 0; k < m.filters.size(); ++k)
      if (m.filters[k].type == FILTER_MESH && m.filters[k].mesh == g.mesh) mesh_filter = static_cast<int>(k);
    if (mesh_filter < 0) {
      HFilter f;
      f.id = fid++;
      f.type = FILTER_MESH;
      f.mesh = g.mesh;
      f.nbins = static_cast<int>(m.meshes[g.mesh].n_bins());
      mesh_filter = static_cast<int>(m.filters.size());
      m.filters.push_back(f);
    }
    HFilter fe;
    fe.id = fid++;
    fe.type = FILTER_ENERGY;
    fe.mesh = -1;
    fe.bins = m.weight_windows[g.ww].ebounds;
    fe.nbins = static_cast<int>(fe.bins.size()) - 1;
    m.filters.push_back(fe);
    HFilter fp;
    fp.id = fid++;
    fp.type = FILTER_PARTICLE;
    fp.mesh = -1;
    fp.nbins = 1;
    m.filters.push_back(fp);
    HTally t;
    int tid = 1;
    for (const auto& tt : m.tallies) tid = std::max(tid, tt.id + 1);
    t.id = tid;
    t.filters = {mesh_filter, static_cast<int>(m.filters.size()) - 2, static_cast<int>(m.filters.size()) - 1};
    t.scores = {SCORE_FLUX};
    t.generated = true;
    t.strides.assign(3, 1);
    int64_t stride = 1;
    for (int i = 2; i >= 0; --i) {
      t.strides[i] = static_cast<int>(stride);
      stride *= m.filters[t.filters[i]].nbins;
    }
    t.n_filter_bins = stride;
    t.results.assign(static_cast<size_t>(stride) * 3, 0.0);
    g.tally = static_cast<int>(m.tallies.size());
    m.tallies.push_back(std::move(t));
    if (g.on_the_fly) m.ww_on = true;
  }
}

// WeightWindows::update_weights (MAGIC), src/weight_windows.cpp:502-755:
// on the device while a simulation holds the tallies there (the first
// window set, the one the transport uses), else on the host arrays.
int update_magic(HModel& m, int ww_idx, int tally_idx, const std::string& value, double threshold, double ratio)
{
  if (ww_idx < 0 || ww_idx >= static_cast<int>(m.weight_windows.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in weight windows array is out of bounds.");
  if (tally_idx < 0 || tally_idx >= static_cast<int>(m.tallies.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in tallies array is out of bounds.");
  if (value != "mean" && value != "rel_err")
    return fail(OPENMC_E_INVALID_ARGUMENT, "Invalid value '" + value + "' specified for weight window generation.");
  HWeightWindows& w = m.weight_windows[ww_idx];
  HTally& t = m.tallies[tally_idx];
  int score_index = -1;
  for (size_t k = 0; k < t.scores.size(); ++k)
    if (t.scores[k] == SCORE_FLUX) score_index = static_cast<int>(k);
  if (score_index < 0) return fail(OPENMC_E_INVALID_ARGUMENT, "A 'flux' score is required for weight window generation.");
  int mesh_pos = -1, energy_pos = -1;
  for (size_t i = 0; i < t.filters.size(); ++i) {
    const HFilter& f = m.filters[t.filters[i]];
    if (f.type == FILTER_MESH) {
      if (f.mesh != w.mesh) return fail(OPENMC_E_INVALID_ARGUMENT, "tally mesh differs from the weight-window mesh");
      mesh_pos = static_cast<int>(i);
    } else if (f.type == FILTER_ENERGY) {
      if (f.bins != w.ebounds) return fail(OPENMC_E_INVALID_ARGUMENT, "tally energy bins differ from the weight-window energy bounds");
      energy_pos = static_cast<int>(i);
    }
  }
  if (mesh_pos < 0) return fail(OPENMC_E_INVALID_ARGUMENT, "tally needs a mesh filter for weight window generation");
  const int e_bins = static_cast<int>(w.ebounds.size()) - 1;
  const int64_t mesh_bins = m.meshes[w.mesh].n_bins();
  const int ns = static_cast<int>(t.scores.size());
  const int n = t.n_realizations;
  const HMesh& mesh = m.meshes[w.mesh];
  double vol = 1.0;
  for (int i = 0; i < mesh.ndim; ++i) vol *= mesh.width[i];
  if (S().gpu && ww_idx == 0) {
    // on the device, from the device's tally sums, into the transport's own
    // window arrays (the host arrays receive a copy)
    MagicArgs a;
    a.tally = tally_idx;
    a.score = score_index;
    a.n_scores = ns;
    a.stride_mesh = t.strides[mesh_pos];
    a.stride_energy = energy_pos >= 0 ? t.strides[energy_pos] : -1;
    a.e_bins = e_bins;
    a.mesh_bins = mesh_bins;
    a.n = n;
    a.volume = vol;
    a.rel_err = value == "rel_err" ? 1 : 0;
    a.threshold = threshold;
    a.ratio = ratio;
    gpu_update_magic(S().gpu, a, w.lower.data(), w.upper.data());
    return 0;
  }
  if (S().gpu) gpu_fetch_tallies(S().gpu, m);
  auto idx = [&](int e, int64_t mb) {
    int64_t k = mb * t.strides[mesh_pos];
    if (energy_pos >= 0) k += static_cast<int64_t>(e) * t.strides[energy_pos];
    return (k * ns + score_index) * 3;
  };
  std::vector<double>& nb = w.lower;
  std::vector<double>& rel = w.upper;
  for (int e = 0; e < e_bins; e++) {
    for (int64_t mb = 0; mb < mesh_bins; mb++) {
      int64_t k = e * mesh_bins + mb;
      double sum = t.results[idx(e, mb) + 1];
      double sum_sq = t.results[idx(e, mb) + 2];
      nb[k] = sum / n;
      if (sum > 0.0) {
        double mean_val = nb[k];
        double variance = (sum_sq / n - mean_val * mean_val) / (n - 1);
        rel[k] = std::sqrt(variance) / mean_val;
      } else {
        rel[k] = std::numeric_limits<double>::max();
      }
      if (value == "rel_err") nb[k] = 1.0 / rel[k];
    }
  }
  for (int e = 0; e < e_bins; e++)
    for (int64_t mb = 0; mb < mesh_bins; mb++) nb[e * mesh_bins + mb] /= vol;
  for (int e = 0; e < e_bins; e++) {
    double group_max = 0.0;
    for (int64_t mb = 0; mb < mesh_bins; mb++)
      if (nb[e * mesh_bins + mb] > group_max) group_max = nb[e * mesh_bins + mb];
    if (group_max > 0.0) {
      double norm_factor = 1.0 / (2.0 * group_max);
      for (int64_t mb = 0; mb < mesh_bins; mb++) nb[e * mesh_bins + mb] *= norm_factor;
    }
  }
  for (int e = 0; e < e_bins; e++) {
    for (int64_t mb = 0; mb < mesh_bins; mb++) {
      int64_t k = e * mesh_bins + mb;
      double sum = t.results[idx(e, mb) + 1];
      if (sum <= 0.0) nb[k] = -1.0;
      else if (rel[k] > threshold) nb[k] = -1.0;
      w.upper[k] = ratio * w.lower[k];
    }
  }
  if (S().gpu && ww_idx == 0) gpu_set_ww_bounds(S().gpu, w.lower.data(), w.upper.data(), static_cast<long long>(w.lower.size()));
  return 0;
}

}  // namespace

namespace omc {
// The loaded model (nullptr before openmc_init) and the error setter, for
// the model getters and off-path entry points of capi_model.cpp.
HModel* capi_model() { return S().model_loaded ? &S().model : nullptr; }
int capi_fail(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace omc

namespace {

// One eigenvalue generation's end: src/simulation.cpp:522-570
// finalize_generation (global tallies, fission-bank sort and comb on the
// device, generation and average k), then src/tallies/tally.cpp:1059-1100
// accumulate_tallies and src/simulation.cpp:414-418 (global tallies and
// realizations reset after an inactive batch).
void finish_generation(State& s, HModel& m, const BatchStats& st, bool active)
{
  auto& gt = s.global_tallies;  // [K_COLLISION, K_ABSORPTION, K_TRACKLENGTH, LEAKAGE][VALUE, SUM, SUM_SQ]
  const double keff_generation_start = gt[6];
  GenerationStats g = gpu_finish_generation(s.gpu, current_batch);
  s.fission_sites = g.fission_sites;
  gt[0] += g.k_col;
  gt[3] += g.k_abs;
  gt[6] += g.k_tra;
  gt[9] += st.leakage;
  // src/eigenvalue.cpp:50-84 calculate_generation_keff
  double kg = gt[6] - keff_generation_start;
  kg /= m.n_particles;
  s.k_generation.push_back(kg);
  // src/eigenvalue.cpp:367-418 calculate_average_keff (one generation per
  // batch, no confidence-interval t-value)
  const int i = static_cast<int>(s.k_generation.size()) - 1;
  const int n = active ? n_realizations + 1 : 0;
  if (n <= 0) {
    keff = s.k_generation[i];
  } else {
    s.k_sum[0] += s.k_generation[i];
    s.k_sum[1] += std::pow(s.k_generation[i], 2);
    keff = s.k_sum[0] / n;
    if (n > 1) {
      const double t_value = 1.0;
      keff_std = t_value * std::sqrt((s.k_sum[1] / n - std::pow(keff, 2)) / (n - 1));
      if (!std::isfinite(keff_std)) keff_std = 0.0;
    }
  }
  gpu_set_keff(s.gpu, keff);
  // accumulate_tallies: global tallies per unit source weight
  ++n_realizations;
  const double tw = st.total_weight;
  if (active) {
    const double k_col = gt[0] / tw, k_abs = gt[3] / tw, k_tra = gt[6] / tw;
    s.k_col_abs += k_col * k_abs;
    s.k_col_tra += k_col * k_tra;
    s.k_abs_tra += k_abs * k_tra;
  }
  for (int t = 0; t < 4; ++t) {
    const double val = gt[3 * t] / tw;
    gt[3 * t] = 0.0;
    gt[3 * t + 1] += val;
    gt[3 * t + 2] += val * val;
  }
  if (!active) {
    std::fill(gt.begin(), gt.end(), 0.0);
    n_realizations = 0;
  }
}

int check_device_errors(const BatchStats& st)
{
  HModel& m = S().model;
  n_lost_particles += st.n_lost;
  if (st.error & ERR_SECONDARY_OVERFLOW)
    return fail(OPENMC_E_ALLOCATE, "The secondary particle pool on the GPU is full; raise openmc_gb300_secondary_capacity.");
  if (st.error & ERR_NO_NUCLIDE) return fail(OPENMC_E_PHYSICS, "Did not sample any nuclide during collision.");
  if (st.error & ERR_REJECTION)
    return fail(OPENMC_E_INVALID_ARGUMENT, "Too few source sites satisfied the constraints.");
  if (st.error & ERR_ITERATIONS) return fail(OPENMC_E_UNASSIGNED, "Event loop exceeded its iteration limit.");
  double n_sim = static_cast<double>(current_batch) * m.n_particles;
  if (n_lost_particles > 0 && n_lost_particles >= m.max_lost_particles &&
      n_lost_particles >= m.rel_max_lost_particles * n_sim)
    return fail(OPENMC_E_GEOMETRY, "Maximum number of lost particles has been reached.");
  return 0;
}

}  // namespace

extern "C" {

namespace {
void write_statepoint(const std::string& path);
std::string default_statepoint_name(const HModel& m);
}  // namespace

// src/initialize.cpp:45-138, 215-330 (arguments: [-e] [-n N] [-s N] [path])
int openmc_init(int argc, char* argv[], const void* intracomm)
{
  (void)intracomm;
  try {
    State& s = S();
    if (s.gpu) {
      gpu_destroy(s.gpu);
      s.gpu = nullptr;
    }
    s = State();
    std::string path = ".";
    bool cli_event = false;
    int64_t cli_particles = -1;
    for (int i = 1; i < argc; ++i) {
      std::string a = argv[i] ? argv[i] : "";
      if (a == "-e" || a == "--event") cli_event = true;
      else if ((a == "-n" || a == "--particles") && i + 1 < argc) cli_particles = std::stoll(argv[++i]);
      else if ((a == "-s" || a == "--threads") && i + 1 < argc) ++i;
      else if (a == "-r" || a == "--restart") return fail(OPENMC_E_INVALID_ARGUMENT, "restart runs are not supported");
      else if (a == "-p" || a == "--plot" || a == "-c" || a == "--volume" || a == "-t" || a == "--track")
        return fail(OPENMC_E_INVALID_ARGUMENT, "run mode '" + a + "' is not supported");
      else if (!a.empty() && a[0] != '-') path = a;
    }
    load_model(path, s.model);
    finalize_model(s.model);
    if (cli_particles > 0) s.model.n_particles = cli_particles;
    if (cli_event) s.model.event_based = true;
    setup_generators(s.model);
    s.seed = s.model.seed;
    s.stride = s.model.stride;
    s.model_loaded = true;
    s.global_tallies.assign(12, 0.0);
    sync_globals_from_model();
    current_batch = 0;
    n_realizations = 0;
    n_lost_particles = 0;
    initialized = false;
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_INVALID_ARGUMENT, e.what());
  }
}

// src/simulation.cpp:75-166
int openmc_simulation_init()
{
  State& s = S();
  if (initialized) return 0;
  if (!s.model_loaded) return fail(OPENMC_E_ALLOCATE, "OpenMC has not been initialized.");
  try {
    HModel& m = s.model;
    // settings Python may have changed between init and simulation_init
    m.n_particles = n_particles;
    m.n_inactive = n_inactive;
    m.event_based = event_based;
    m.ww_on = weight_windows_on;
    m.seed = s.seed;
    m.stride = s.stride;
    if (m.n_batches <= m.n_inactive) return fail(OPENMC_E_INVALID_ARGUMENT, "Number of active batches must be greater than zero.");
    GpuOptions opt;
    opt.in_flight = openmc_gb300_in_flight > 0 ? openmc_gb300_in_flight : m.max_particles_in_flight;
    opt.xs_fp32 = openmc_gb300_xs_fp32 >= 0 ? openmc_gb300_xs_fp32 != 0 : m.xs_precision == 32;
    opt.sort = openmc_gb300_sort != 0;
    opt.tail_threshold = openmc_gb300_tail_threshold;
    opt.secondary_cap = openmc_gb300_secondary_capacity;
    opt.split_slots = openmc_gb300_split_to_slots;
    opt.max_levels = openmc_gb300_max_levels;
    opt.stage_tables = openmc_gb300_stage_tables;
    opt.fuse = openmc_gb300_fuse;
    opt.contract = openmc_gb300_contract;
    opt.defer_tally = openmc_gb300_defer_tally;
    if (m.ww_on && m.weight_windows.empty()) return fail(OPENMC_E_INVALID_ARGUMENT, "weight windows are on but none are defined");
    s.gpu = gpu_create(m, opt);
    if (s.trace_hist > 0) gpu_set_trace(s.gpu, s.trace_hist, s.trace_cap, openmc_gb300_trace_batch, openmc_gb300_trace_first);
    gpu_reset_tallies(s.gpu, m);
    std::fill(s.global_tallies.begin(), s.global_tallies.end(), 0.0);
    s.k_generation.clear();
    s.k_sum[0] = s.k_sum[1] = 0.0;
    s.k_col_abs = s.k_col_tra = s.k_abs_tra = 0.0;
    s.fission_sites = 0;
    keff = 1.0;
    keff_std = 0.0;
    current_batch = 0;
    n_realizations = 0;
    n_lost_particles = 0;
    s.time_active = s.time_inactive = s.time_wall_active = 0.0;
    s.n_batches_run = 0;
    initialized = true;
    return 0;
  } catch (const std::exception& e) {
    if (s.gpu) {
      gpu_destroy(s.gpu);
      s.gpu = nullptr;
    }
    return fail(OPENMC_E_ALLOCATE, e.what());
  }
}

// src/simulation.cpp:232-280 (status 0 normal, 1 reached max batches)
int openmc_next_batch(int* status)
{
  State& s = S();
  if (!initialized) return fail(OPENMC_E_ALLOCATE, "Simulation has not been initialized yet.");
  HModel& m = s.model;
  if (status) *status = 0;
  if (current_batch >= m.n_batches) {
    if (status) *status = 1;
    return 0;
  }
  try {
    ++current_batch;
    bool active = current_batch > m.n_inactive;
    auto t0 = std::chrono::steady_clock::now();
    BatchStats st = openmc_gb300_profile_next ? gpu_run_batch_profiled(s.gpu, m, current_batch, active)
                                              : gpu_run_batch(s.gpu, m, current_batch, active);
    if (openmc_gb300_profile_next == 1) openmc_gb300_profile_next = 0;
    auto t1 = std::chrono::steady_clock::now();
    s.last = st;
    s.n_batches_run++;
    if (active) {
      s.time_active += st.ms * 1e-3;
      s.time_wall_active += std::chrono::duration<double>(t1 - t0).count();
    } else {
      s.time_inactive += st.ms * 1e-3;
    }
    if (int rc = check_device_errors(st)) return rc;
    if (m.eigenvalue) {
      finish_generation(s, m, st, active);
    } else if (active) {
      ++n_realizations;
      // global leakage tally normalised by total source weight (tally.cpp:1059-1100)
      double val = st.leakage / st.total_weight;
      s.global_tallies[9 + 1] += val;
      s.global_tallies[9 + 2] += val * val;
    }
    if (active) {
      // weight-window generators (src/weight_windows.cpp:967-994)
      bool need = false;
      for (const auto& g : m.ww_generators) need = need || g.tally >= 0;
      if (need) {
        for (const auto& g : m.ww_generators) {
          const HTally& t = m.tallies[g.tally];
          if (g.max_realizations < t.n_realizations || t.n_realizations % g.update_interval != 0) continue;
          if (int rc = update_magic(m, g.ww, g.tally, g.value, g.threshold, g.ratio)) return rc;
        }
      }
    }
    if (current_batch >= m.n_batches) {
      // src/simulation.cpp:432-441: the last batch is a statepoint batch
      gpu_fetch_tallies(s.gpu, m);
      write_statepoint(default_statepoint_name(m));
    }
    if (status && current_batch >= m.n_batches) *status = 1;
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

namespace {

// Shortest round-trip decimal form of a double, as the reference's fmt "{}".
std::string shortest(double v)
{
  char buf[64];
  auto r = std::to_chars(buf, buf + sizeof(buf), v);
  return std::string(buf, r.ptr);
}

// " ====...>     TEXT     <====...", src/output.cpp:103-125
std::string header_line(const std::string& msg)
{
  const int len = static_cast<int>(msg.size());
  const int n_prefix = (63 - len) / 2;
  const int n_suffix = n_prefix + ((len % 2) == 0 ? 1 : 0);
  std::string upper(msg);
  std::transform(upper.begin(), upper.end(), upper.begin(), [](unsigned char c) { return std::toupper(c); });
  return " " + std::string(std::max(n_prefix, 0), '=') + ">     " + upper + "     <" +
         std::string(std::max(n_suffix, 0), '=');
}

std::string filter_label(const HModel& m, const HFilter& f, int bin)
{
  switch (f.type) {
  case FILTER_MESH: {
    // src/mesh.cpp:604-615 bin_label, x index fastest, 1-based
    const HMesh& mesh = m.meshes[f.mesh];
    int ijk[3] = {0, 0, 0};
    int rem = bin;
    for (int i = 0; i < mesh.ndim; ++i) {
      ijk[i] = rem % mesh.shape[i] + 1;
      rem /= mesh.shape[i];
    }
    if (mesh.ndim > 2) return "Mesh Index (" + std::to_string(ijk[0]) + ", " + std::to_string(ijk[1]) + ", " +
                              std::to_string(ijk[2]) + ")";
    if (mesh.ndim > 1) return "Mesh Index (" + std::to_string(ijk[0]) + ", " + std::to_string(ijk[1]) + ")";
    return "Mesh Index (" + std::to_string(ijk[0]) + ")";
  }
  case FILTER_ENERGY:  // src/tallies/filter_energy.cpp:89-92
    return "Incoming Energy [" + shortest(f.bins[bin]) + ", " + shortest(f.bins[bin + 1]) + ")";
  case FILTER_PARTICLE:  // src/tallies/filter_particle.cpp:55-59
    return "Particle: neutron";
  case FILTER_CELL:  // src/tallies/filter_cell.cpp:69-72
    return "Cell " + std::to_string(m.cells[f.ids[bin]].id);
  default:  // src/tallies/filter_material.cpp
    return "Material " + std::to_string(m.materials[f.ids[bin]].id);
  }
}

// src/output.cpp:605-720 write_tallies: every filter-bin combination (last
// filter fastest), a filter's label where its bin starts, "Total Material",
// then "score  mean +/- standard deviation of the mean" (t-value 1).
void write_tallies(const HModel& m)
{
  if (m.tallies.empty() || !m.output_tallies) return;
  std::string dir = m.path_output.empty() ? std::string(".") : m.path_output;
  std::ofstream out(dir + "/tallies.out", std::ios::out | std::ios::trunc);
  if (!out) return;
  static const char* score_name[] = {"Flux", "Total Reaction Rate", "Absorption Rate"};
  char line[256];
  for (const auto& t : m.tallies) {
    std::string title = "TALLY " + std::to_string(t.id);
    if (!t.name.empty()) title += ": " + t.name;
    out << header_line(title) << "\n\n";
    const int nf = static_cast<int>(t.filters.size());
    const int ns = static_cast<int>(t.scores.size());
    const int n = t.n_realizations;
    for (int64_t index = 0; index < t.n_filter_bins; ++index) {
      int indent = 0;
      for (int i = 0; i < nf; ++i) {
        if (index % t.strides[i] == 0) {
          const HFilter& f = m.filters[t.filters[i]];
          const int bin = static_cast<int>((index / t.strides[i]) % f.nbins);
          out << std::string(indent + 1, ' ') << filter_label(m, f, bin) << "\n";
        }
        indent += 2;
      }
      out << std::string(indent + 1, ' ') << "Total Material\n";
      indent += 2;
      for (int s = 0; s < ns; ++s) {
        const double* r = &t.results[(index * ns + s) * 3];
        double mean = n > 0 ? r[1] / n : 0.0;
        double sd = 0.0;
        if (n > 1) sd = std::sqrt(std::max((r[2] / n - mean * mean) / (n - 1), 0.0));
        std::snprintf(line, sizeof(line), "%*s%-36s %.6g +/- %.6g\n", indent + 1, "", score_name[t.scores[s]],
          mean, sd);
        out << line;
      }
    }
  }
}

// A fixed-length string array dataset ("char[][]" of the file formats)
h5::Value strings(const std::vector<std::string>& v)
{
  h5::Value out;
  out.kind = 's';
  out.size = 1;
  for (const auto& x : v) out.size = std::max(out.size, x.size());
  out.shape = {v.size()};
  out.bytes.assign(out.size * v.size(), 0);
  for (size_t k = 0; k < v.size(); ++k) std::copy(v[k].begin(), v[k].end(), out.bytes.begin() + k * out.size);
  return out;
}

h5::Value int_array(const std::vector<int>& v)
{
  return h5::array(std::vector<long long>(v.begin(), v.end()));
}

// src/state_point.cpp:36-357 openmc_statepoint_write in the statepoint file
// format 18.1 (docs/source/io_formats/statepoint.rst): run parameters,
// k-effective results of an eigenvalue run, global tallies, and every
// tally with its meshes and filters and its accumulated (SUM, SUM_SQ)
// results.  No source bank is written (source_present 0).
void write_statepoint(const std::string& path)
{
  State& s = S();
  const HModel& m = s.model;
  h5::WNode root;
  root.attrs["filetype"] = h5::string("statepoint");
  root.attrs["version"] = h5::array(std::vector<long long> {18, 1});
  root.attrs["openmc_version"] = h5::array(std::vector<long long> {0, 15, 0});
  root.attrs["git_sha1"] = h5::string(std::string(40, '0'));
  {
    std::time_t t = std::time(nullptr);
    char buf[64];
    std::strftime(buf, sizeof(buf), "%Y-%m-%d %H:%M:%S", std::localtime(&t));
    root.attrs["date_and_time"] = h5::string(buf);
  }
  root.attrs["path"] = h5::string(m.path_output);
  root.attrs["tallies_present"] = h5::scalar(static_cast<long long>(m.tallies.empty() ? 0 : 1));
  root.attrs["source_present"] = h5::scalar(0LL);
  root.dataset("seed", h5::scalar(static_cast<long long>(s.seed)));
  {
    h5::Value st = h5::scalar(static_cast<long long>(s.stride));
    st.kind = 'u';
    root.dataset("stride", st);
  }
  root.dataset("energy_mode", h5::string("continuous-energy"));
  root.dataset("run_mode", h5::string(m.eigenvalue ? "eigenvalue" : "fixed source"));
  root.dataset("n_particles", h5::scalar(static_cast<long long>(m.n_particles)));
  root.dataset("n_batches", h5::scalar(static_cast<long long>(m.n_batches)));
  root.dataset("current_batch", h5::scalar(static_cast<long long>(current_batch)));
  if (m.eigenvalue) {
    root.dataset("n_inactive", h5::scalar(static_cast<long long>(m.n_inactive)));
    root.dataset("generations_per_batch", h5::scalar(1LL));
    root.dataset("k_generation", h5::array(s.k_generation));
    root.dataset("entropy", h5::array(std::vector<double> {}));
    root.dataset("k_col_abs", h5::scalar(s.k_col_abs));
    root.dataset("k_col_tra", h5::scalar(s.k_col_tra));
    root.dataset("k_abs_tra", h5::scalar(s.k_abs_tra));
    double kc[2];
    openmc_get_keff(kc);
    root.dataset("k_combined", h5::array(std::vector<double> {kc[0], kc[1]}));
  }
  root.dataset("n_realizations", h5::scalar(static_cast<long long>(n_realizations)));
  {
    std::vector<double> gt;
    for (int t = 0; t < 4; ++t) {
      gt.push_back(s.global_tallies[3 * t + 1]);
      gt.push_back(s.global_tallies[3 * t + 2]);
    }
    root.dataset("global_tallies", h5::array(gt, {4, 2}));
  }
  h5::WNode& tg = root.group_at("tallies");
  std::vector<int> tally_ids, mesh_ids, filter_ids;
  for (const auto& t : m.tallies)
    if (!t.generated) tally_ids.push_back(t.id);
  tg.attrs["n_tallies"] = h5::scalar(static_cast<long long>(tally_ids.size()));
  tg.attrs["ids"] = int_array(tally_ids);
  h5::WNode& mg = tg.group_at("meshes");
  for (const auto& mesh : m.meshes) {
    mesh_ids.push_back(mesh.id);
    h5::WNode& g = mg.group_at("mesh " + std::to_string(mesh.id));
    g.attrs["id"] = h5::scalar(static_cast<long long>(mesh.id));
    g.dataset("name", h5::string(""));
    g.dataset("type", h5::string("regular"));
    g.dataset("dimension", int_array(std::vector<int>(mesh.shape, mesh.shape + mesh.ndim)));
    g.dataset("lower_left", h5::array(std::vector<double>(mesh.ll, mesh.ll + mesh.ndim)));
    g.dataset("upper_right", h5::array(std::vector<double>(mesh.ur, mesh.ur + mesh.ndim)));
    g.dataset("width", h5::array(std::vector<double>(mesh.width, mesh.width + mesh.ndim)));
  }
  mg.attrs["n_meshes"] = h5::scalar(static_cast<long long>(mesh_ids.size()));
  mg.attrs["ids"] = int_array(mesh_ids);
  h5::WNode& fg = tg.group_at("filters");
  static const char* ftype[] = {"mesh", "energy", "particle", "cell", "material"};
  for (const auto& f : m.filters) {
    filter_ids.push_back(f.id);
    h5::WNode& g = fg.group_at("filter " + std::to_string(f.id));
    g.dataset("type", h5::string(ftype[f.type]));
    g.dataset("n_bins", h5::scalar(static_cast<long long>(f.nbins)));
    if (f.type == FILTER_MESH) {
      g.dataset("bins", h5::scalar(static_cast<long long>(m.meshes[f.mesh].id)));
    } else if (f.type == FILTER_ENERGY) {
      g.dataset("bins", h5::array(f.bins));
    } else if (f.type == FILTER_CELL || f.type == FILTER_MATERIAL) {
      std::vector<int> ids;
      for (int i : f.ids) ids.push_back(f.type == FILTER_CELL ? m.cells[i].id : m.materials[i].id);
      g.dataset("bins", int_array(ids));
    } else {
      g.dataset("bins", strings({"neutron"}));
    }
  }
  fg.attrs["n_filters"] = h5::scalar(static_cast<long long>(filter_ids.size()));
  fg.attrs["ids"] = int_array(filter_ids);
  static const char* sname[] = {"flux", "total", "absorption"};
  for (const auto& t : m.tallies) {
    if (t.generated) continue;
    h5::WNode& g = tg.group_at("tally " + std::to_string(t.id));
    g.attrs["internal"] = h5::scalar(0LL);
    g.attrs["multiply_density"] = h5::scalar(1LL);
    g.attrs["higher_moments"] = h5::scalar(0LL);
    g.dataset("n_realizations", h5::scalar(static_cast<long long>(t.n_realizations)));
    g.dataset("n_filters", h5::scalar(static_cast<long long>(t.filters.size())));
    std::vector<int> fids;
    for (int fi : t.filters) fids.push_back(m.filters[fi].id);
    g.dataset("filters", int_array(fids));
    g.dataset("nuclides", strings({"total"}));
    g.dataset("estimator", h5::string(t.estimator == EST_COLLISION ? "collision" : "tracklength"));
    g.dataset("n_score_bins", h5::scalar(static_cast<long long>(t.scores.size())));
    std::vector<std::string> sc;
    for (int k : t.scores) sc.push_back(sname[k]);
    g.dataset("score_bins", strings(sc));
    const int64_t ns = static_cast<int64_t>(t.scores.size());
    std::vector<double> res(static_cast<size_t>(t.n_filter_bins * ns * 2));
    for (int64_t k = 0; k < t.n_filter_bins * ns && 3 * k + 2 < static_cast<int64_t>(t.results.size()); ++k) {
      res[2 * k] = t.results[3 * k + 1];
      res[2 * k + 1] = t.results[3 * k + 2];
    }
    g.dataset("results", h5::array(res, {static_cast<uint64_t>(t.n_filter_bins), static_cast<uint64_t>(ns), 2}));
  }
  h5::WNode& rt = root.group_at("runtime");
  rt.dataset("simulation", h5::scalar(s.time_active + s.time_inactive));
  rt.dataset("transport", h5::scalar(s.time_active + s.time_inactive));
  rt.dataset("inactive batches", h5::scalar(s.time_inactive));
  rt.dataset("active batches", h5::scalar(s.time_active));
  h5::write(path, root);
}

// The default statepoint name: <output path>/statepoint.<batch, zero-padded
// to the width of n_batches>.h5 (src/state_point.cpp:46-51)
std::string default_statepoint_name(const HModel& m)
{
  const std::string dir = m.path_output.empty() ? std::string(".") : m.path_output;
  const int w = static_cast<int>(std::to_string(m.n_batches).size());
  char buf[32];
  std::snprintf(buf, sizeof(buf), "%0*d", w, current_batch);
  return dir + "/statepoint." + buf + ".h5";
}

}  // namespace

// src/state_point.cpp:36-357: tallies are copied from the device first;
// filename null gives the default name
int openmc_statepoint_write(const char* filename, bool* write_source)
{
  (void)write_source;  // no source bank is written
  State& s = S();
  if (!s.model_loaded) return fail(OPENMC_E_ALLOCATE, "OpenMC has not been initialized.");
  try {
    if (s.gpu) gpu_fetch_tallies(s.gpu, s.model);
    write_statepoint(filename ? std::string(filename) : default_statepoint_name(s.model));
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

int openmc_simulation_finalize()
{
  State& s = S();
  if (!initialized) return 0;
  try {
    gpu_fetch_tallies(s.gpu, s.model);
    gpu_destroy(s.gpu);
    s.gpu = nullptr;
    initialized = false;
    write_tallies(s.model);  // src/simulation.cpp:183-185
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

// src/simulation.cpp:53-73
int openmc_run()
{
  if (int rc = openmc_simulation_init()) return rc;
  int status = 0;
  while (status == 0) {
    if (int rc = openmc_next_batch(&status)) {
      openmc_simulation_finalize();
      return rc;
    }
  }
  return openmc_simulation_finalize();
}

int openmc_finalize()
{
  State& s = S();
  if (s.gpu) {
    gpu_destroy(s.gpu);
    s.gpu = nullptr;
  }
  s = State();
  initialized = false;
  current_batch = 0;
  n_realizations = 0;
  n_particles = 0;
  n_lost_particles = 0;
  event_based = false;
  return 0;
}

int openmc_reset()
{
  State& s = S();
  for (auto& t : s.model.tallies) {
    t.n_realizations = 0;
    std::fill(t.results.begin(), t.results.end(), 0.0);
  }
  try {
    if (s.gpu) gpu_reset_tallies(s.gpu, s.model);
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
  std::fill(s.global_tallies.begin(), s.global_tallies.end(), 0.0);
  s.time_active = s.time_inactive = s.time_wall_active = 0.0;
  n_realizations = 0;
  return 0;
}

int openmc_hard_reset()
{
  openmc_reset();
  S().seed = 1;
  return 0;
}

int openmc_reset_timers()
{
  State& s = S();
  s.time_active = s.time_inactive = s.time_wall_active = 0.0;
  return 0;
}

// src/random_lcg.cpp:126-144
int64_t openmc_get_seed() { return S().seed; }
void openmc_set_seed(int64_t new_seed) { S().seed = new_seed; }
uint64_t openmc_get_stride() { return S().stride; }
void openmc_set_stride(uint64_t new_stride) { S().stride = new_stride; }

// src/tallies/tally.cpp:1554-1575: borrowed pointer to [bins][scores][3]
int openmc_tally_results(int32_t index, double** ptr, size_t shape_[3])
{
  State& s = S();
  if (index < 0 || index >= static_cast<int32_t>(s.model.tallies.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in tallies array is out of bounds.");
  try {
    if (s.gpu) gpu_fetch_tallies(s.gpu, s.model);
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
  HTally& t = s.model.tallies[index];
  *ptr = t.results.data();
  shape_[0] = static_cast<size_t>(t.n_filter_bins);
  shape_[1] = t.scores.size();
  shape_[2] = 3;
  return 0;
}

int openmc_get_tally_index(int32_t id, int32_t* index)
{
  const auto& ts = S().model.tallies;
  for (size_t k = 0; k < ts.size(); ++k)
    if (ts[k].id == id) {
      *index = static_cast<int32_t>(k);
      return 0;
    }
  return fail(OPENMC_E_INVALID_ID, "No tally exists with ID=" + std::to_string(id) + ".");
}

int openmc_tally_get_id(int32_t index, int32_t* id)
{
  const auto& ts = S().model.tallies;
  if (index < 0 || index >= static_cast<int32_t>(ts.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in tallies array is out of bounds.");
  *id = ts[index].id;
  return 0;
}

int openmc_tally_get_n_realizations(int32_t index, int32_t* n)
{
  const auto& ts = S().model.tallies;
  if (index < 0 || index >= static_cast<int32_t>(ts.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in tallies array is out of bounds.");
  *n = ts[index].n_realizations;
  return 0;
}

size_t tallies_size() { return S().model.tallies.size(); }

// global tallies [4][3] (K_COLLISION, K_ABSORPTION, K_TRACKLENGTH, LEAKAGE)
int openmc_global_tallies(double** ptr)
{
  *ptr = S().global_tallies.data();
  return 0;
}

// ------------------------------------------------------ weight windows
// src/eigenvalue.cpp:420-579 openmc_get_keff: up to three realizations the
// average k and its spread (infinite up to one realization; a fixed-source
// run keeps k = 1); beyond, the combination of the collision, absorption and
// track-length estimators weighted by their covariances (Urbatsch), or of
// two of them when two estimators coincide.
int openmc_get_keff(double* k_combined)
{
  const State& s = S();
  k_combined[0] = 0.0;
  k_combined[1] = 0.0;
  if (n_realizations <= 3) {
    k_combined[0] = keff;
    k_combined[1] = keff_std;
    if (n_realizations <= 1) k_combined[1] = std::numeric_limits<double>::infinity();
    return 0;
  }
  const int64_t n = n_realizations;
  const auto& gt = s.global_tallies;
  double kv[3], cov[3][3];
  for (int e = 0; e < 3; ++e) kv[e] = gt[3 * e + 1] / n;
  for (int e = 0; e < 3; ++e) cov[e][e] = (gt[3 * e + 2] - n * kv[e] * kv[e]) / (n - 1);
  cov[0][1] = cov[1][0] = (s.k_col_abs - n * kv[0] * kv[1]) / (n - 1);
  cov[0][2] = cov[2][0] = (s.k_col_tra - n * kv[0] * kv[2]) / (n - 1);
  cov[1][2] = cov[2][1] = (s.k_abs_tra - n * kv[1] * kv[2]) / (n - 1);
  const double rel = 1e-5;  // FP_REL_PRECISION
  auto same = [&](int a, int b) {
    return std::abs(kv[a] - kv[b]) / kv[a] < rel && std::abs(cov[a][a] - cov[b][b]) / cov[a][a] < rel;
  };
  int i = 0, j = 0;
  bool use_three = false;
  if (same(0, 1)) {
    i = 0;
    j = 2;
  } else if (same(0, 2)) {
    i = 0;
    j = 1;
  } else if (same(1, 2)) {
    i = 0;
    j = 1;
  } else {
    use_three = true;
  }
  if (use_three) {
    double g = 0.0;
    double S3[3] = {0.0, 0.0, 0.0};
    const int perm[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};  // (i, j, k) for l = 0, 1, 2
    for (int l = 0; l < 3; ++l) {
      const int a = perm[l][0], b = perm[l][1], c = perm[l][2];
      const double f = cov[b][b] * (cov[c][c] - cov[a][c]) - cov[c][c] * cov[a][b] +
                       cov[b][c] * (cov[a][b] + cov[a][c] - cov[b][c]);
      S3[0] += f * cov[0][l];
      S3[1] += (cov[b][b] + cov[c][c] - 2.0 * cov[b][c]) * kv[l] * kv[l];
      S3[2] += (cov[c][c] + cov[a][b] - cov[b][c] - cov[a][c]) * kv[l] * kv[b];
      k_combined[0] += f * kv[l];
      g += f;
    }
    for (double& v : S3) v *= (n - 1);
    S3[0] *= (n - 1) * (n - 1);
    k_combined[0] /= g;
    g *= (n - 1) * (n - 1);
    k_combined[1] = std::sqrt(S3[0] / (g * n * (n - 3)) * (1 + n * ((S3[1] - 2 * S3[2]) / g)));
  } else {
    const double f = kv[i] - kv[j];
    const double g = cov[i][i] + cov[j][j] - 2.0 * cov[i][j];
    k_combined[0] = kv[i] - (cov[i][i] - cov[i][j]) / g * f;
    k_combined[1] = (cov[i][i] * cov[j][j] - cov[i][j] * cov[i][j]) * (g + n * f * f) / (n * (n - 2) * g * g);
    k_combined[1] = std::sqrt(k_combined[1]);
  }
  return 0;
}

// GB300 extension (no reference counterpart): every generation's
// track-length k (at most n of them; returns how many exist) and the last
// generation's fission-bank size
int openmc_gb300_k_generation(double* k, int n, int64_t* fission_sites)
{
  const State& s = S();
  const int m = static_cast<int>(s.k_generation.size());
  for (int i = 0; i < m && i < n; ++i) k[i] = s.k_generation[i];
  if (fission_sites) *fission_sites = s.fission_sites;
  return m;
}

// src/weight_windows.cpp:1020-1340
size_t openmc_weight_windows_size() { return S().model.weight_windows.size(); }

int openmc_get_weight_windows_index(int32_t id, int32_t* idx)
{
  const auto& w = S().model.weight_windows;
  for (size_t k = 0; k < w.size(); ++k)
    if (w[k].id == id) {
      *idx = static_cast<int32_t>(k);
      return 0;
    }
  return fail(OPENMC_E_INVALID_ID, "Weight windows with ID " + std::to_string(id) + " not found.");
}

int openmc_weight_windows_get_id(int32_t index, int32_t* id)
{
  const auto& w = S().model.weight_windows;
  if (index < 0 || index >= static_cast<int32_t>(w.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in weight windows array is out of bounds.");
  *id = w[index].id;
  return 0;
}

int openmc_weight_windows_get_bounds(int32_t index, const double** lower_bounds, const double** upper_bounds, size_t* size)
{
  auto& w = S().model.weight_windows;
  if (index < 0 || index >= static_cast<int32_t>(w.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in weight windows array is out of bounds.");
  *lower_bounds = w[index].lower.data();
  *upper_bounds = w[index].upper.data();
  *size = w[index].lower.size();
  return 0;
}

int openmc_weight_windows_set_bounds(int32_t index, const double* lower_bounds, const double* upper_bounds, size_t size)
{
  auto& w = S().model.weight_windows;
  if (index < 0 || index >= static_cast<int32_t>(w.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in weight windows array is out of bounds.");
  if (size != w[index].lower.size())
    return fail(OPENMC_E_INVALID_ARGUMENT, "Size of weight window bounds does not match the number of bins.");
  std::copy(lower_bounds, lower_bounds + size, w[index].lower.begin());
  std::copy(upper_bounds, upper_bounds + size, w[index].upper.begin());
  try {
    if (S().gpu && index == 0) gpu_set_ww_bounds(S().gpu, lower_bounds, upper_bounds, static_cast<long long>(size));
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
  return 0;
}

int openmc_weight_windows_get_energy_bounds(int32_t index, const double** e_bounds, size_t* e_bounds_size)
{
  auto& w = S().model.weight_windows;
  if (index < 0 || index >= static_cast<int32_t>(w.size()))
    return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in weight windows array is out of bounds.");
  *e_bounds = w[index].ebounds.data();
  *e_bounds_size = w[index].ebounds.size();
  return 0;
}

int openmc_weight_windows_update_magic(int32_t ww_idx, int32_t tally_idx, const char* value, double threshold, double ratio)
{
  State& s = S();
  try {
    return update_magic(s.model, ww_idx, tally_idx, value ? value : "mean", threshold, ratio);
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

int openmc_weight_windows_get_survival_ratio(int32_t index, double* ratio)
{
  auto& w = S().model.weight_windows;
  if (index < 0 || index >= static_cast<int32_t>(w.size())) return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in weight windows array is out of bounds.");
  *ratio = w[index].survival_ratio;
  return 0;
}

int openmc_weight_windows_get_max_split(int32_t index, int* max_split)
{
  auto& w = S().model.weight_windows;
  if (index < 0 || index >= static_cast<int32_t>(w.size())) return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in weight windows array is out of bounds.");
  *max_split = w[index].max_split;
  return 0;
}

int openmc_weight_windows_get_mesh(int32_t index, int32_t* mesh_idx)
{
  auto& w = S().model.weight_windows;
  if (index < 0 || index >= static_cast<int32_t>(w.size())) return fail(OPENMC_E_OUT_OF_BOUNDS, "Index in weight windows array is out of bounds.");
  *mesh_idx = w[index].mesh;
  return 0;
}

// ------------------------------------------- GB300 extensions (no reference
// counterpart): run statistics, precision and trace controls
int openmc_gb300_last_batch(double* out)
{
  const BatchStats& b = S().last;
  out[0] = b.ms;
  out[1] = b.iterations;
  out[2] = static_cast<double>(b.n_events);
  out[3] = b.total_weight;
  out[4] = b.leakage;
  out[5] = b.n_lost;
  out[6] = static_cast<double>(b.n_done);
  out[7] = b.n_secondaries;
  out[8] = static_cast<double>(b.longest_events);
  out[9] = static_cast<double>(b.longest_id);
  return 0;
}

// [queue phase: xs events, xs recomputations, xs nuclide lookups, mesh
//  segments, collision nuclide lookups, surface events, collisions;
//  tail phase: the same seven; kernel ms x9 (xs, advance, surface, collision,
//  tail, refill, sort, other, track-length tally)]
int openmc_gb300_last_batch_detail(double* out)
{
  const BatchStats& b = S().last;
  for (int a = 0; a < 2; ++a)
    for (int k = 0; k < 7; ++k) out[7 * a + k] = static_cast<double>(b.stat[a][k]);
  for (int k = 0; k < 9; ++k) out[14 + k] = b.kernel_ms[k];
  return 0;
}

int openmc_gb300_timing(double* out)
{
  State& s = S();
  out[0] = s.time_active;
  out[1] = s.time_inactive;
  out[2] = s.time_wall_active;
  int active = std::max(0, current_batch - s.model.n_inactive);
  // src/output.cpp:460-490 calculation rate (active)
  out[3] = s.time_active > 0 ? static_cast<double>(s.model.n_particles) * active / s.time_active : 0.0;
  out[4] = s.gpu ? static_cast<double>(gpu_capacity(s.gpu)) : 0.0;
  return 0;
}

int openmc_gb300_set_trace(int64_t n_hist, int cap)
{
  State& s = S();
  s.trace_hist = n_hist;
  s.trace_cap = cap;
  try {
    if (s.gpu) gpu_set_trace(s.gpu, n_hist, cap, openmc_gb300_trace_batch, openmc_gb300_trace_first);
  } catch (const std::exception& e) {
    return fail(OPENMC_E_ALLOCATE, e.what());
  }
  return 0;
}

int openmc_gb300_get_trace(void* records, int32_t* counts)
{
  State& s = S();
  if (!s.gpu || s.trace_hist <= 0) return fail(OPENMC_E_ALLOCATE, "no trace is being recorded");
  try {
    gpu_get_trace(s.gpu, records, counts);
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
  return 0;
}

int openmc_gb300_set_weight_windows_on(int on)
{
  State& s = S();
  weight_windows_on = on != 0;
  s.model.ww_on = weight_windows_on;
  try {
    if (s.gpu) gpu_set_ww_on(s.gpu, weight_windows_on);
  } catch (const std::exception& e) {
    return fail(OPENMC_E_INVALID_ARGUMENT, e.what());
  }
  return 0;
}

int openmc_gb300_material_xs(int64_t n, const int32_t* material, const double* E, double* total,
                             double* absorption, uint32_t* grid_hash)
{
  State& s = S();
  if (!s.gpu) return fail(OPENMC_E_ALLOCATE, "Simulation has not been initialized.");
  if (n < 0) return fail(OPENMC_E_INVALID_SIZE, "Negative number of lookups.");
  const int n_mat = static_cast<int>(s.model.materials.size());
  for (int64_t i = 0; i < n; ++i)
    if (material[i] < 0 || material[i] >= n_mat) return fail(OPENMC_E_OUT_OF_BOUNDS, "Material index out of range.");
  try {
    gpu_material_xs(s.gpu, n, material, E, total, absorption, grid_hash);
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
  return 0;
}

int openmc_gb300_model_info(int64_t* out)
{
  const HModel& m = S().model;
  out[0] = static_cast<int64_t>(m.nuclides.size());
  out[1] = static_cast<int64_t>(m.materials.size());
  out[2] = static_cast<int64_t>(m.cells.size());
  out[3] = static_cast<int64_t>(m.surfaces.size());
  out[4] = static_cast<int64_t>(m.tallies.size());
  out[5] = m.n_log_bins;
  out[6] = m.n_batches;
  out[7] = m.n_coord_levels;
  return 0;
}

}  // extern "C"
