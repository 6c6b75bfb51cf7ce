// Host-side model of the event-based transport path: what openmc_init builds
// from model.xml (or the separate XML files) and the nuclide library, before
// it is laid out in HBM by the device layer.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace omc {

constexpr int SURF_XPLANE = 0, SURF_YPLANE = 1, SURF_ZPLANE = 2, SURF_XCYL = 3,
              SURF_YCYL = 4, SURF_ZCYL = 5, SURF_SPHERE = 6;
constexpr int BC_TRANSMIT = 0, BC_VACUUM = 1, BC_REFLECT = 2;
constexpr int FILL_MATERIAL = 0, FILL_UNIVERSE = 1, FILL_LATTICE = 2;
constexpr int FILTER_MESH = 0, FILTER_ENERGY = 1, FILTER_PARTICLE = 2, FILTER_CELL = 3, FILTER_MATERIAL = 4;
constexpr int EST_TRACKLENGTH = 0, EST_COLLISION = 1;
constexpr int SCORE_FLUX = 0, SCORE_TOTAL = 1, SCORE_ABSORPTION = 2;
// Region operator tokens, include/openmc/cell.h:31-35
constexpr int32_t OP_LEFT_PAREN = 2147483647;
constexpr int32_t OP_RIGHT_PAREN = OP_LEFT_PAREN - 1;
constexpr int32_t OP_COMPLEMENT = OP_LEFT_PAREN - 2;
constexpr int32_t OP_INTERSECTION = OP_LEFT_PAREN - 3;
constexpr int32_t OP_UNION = OP_LEFT_PAREN - 4;

struct HSurface {
  int id, type, bc;
  double c[4];
};

struct HCell {
  int id, universe, fill_type, fill;
  std::vector<int32_t> expr;  // surface tokens (simple) or postfix (complex)
  bool simple;
  double tr[3];
};

struct HLattice {
  int id;
  int n[3];
  double ll[3], pitch[3];
  bool is3d;
  int outer;
  std::vector<int> univ;  // reference internal order (src/lattice.cpp:220-230)
};

struct HMesh {
  int id, ndim;
  int shape[3];
  double ll[3], ur[3], width[3];
  int64_t n_bins() const { return int64_t(shape[0]) * shape[1] * shape[2]; }
};

struct HFilter {
  int id, type, mesh, nbins;
  std::vector<double> bins;
  std::vector<int> ids;  // cell / material indices of the bins
};

struct HTally {
  int id;
  std::string name;
  int estimator = EST_TRACKLENGTH;
  std::vector<int> filters, strides, scores;
  int64_t n_filter_bins = 1;
  std::vector<double> results;  // [bins][scores][3] host mirror (VALUE, SUM, SUM_SQ)
  int n_realizations = 0;
  bool generated = false;       // created by a weight-window generator
};

struct HNuclide {
  std::string name;
  double awr, kT;
  std::vector<double> energy;
  std::vector<double> total, absorption, elastic;  // create_derived columns + MT2
  std::vector<double> fission, nu_fission;         // create_derived columns (zero without MT 18)
  std::vector<int> grid_index;                     // [M+1]
  // MT 18 prompt neutron product: yield polynomial (increasing powers of E),
  // spectrum 1 Maxwell (sp[0] = theta) or 2 Watt (sp = a, b), restriction
  // energy u; isotropic emission
  bool fissionable = false;
  double nu_c[2] = {0.0, 0.0};
  int spectrum = 0;
  double sp[2] = {0.0, 0.0};
  double u = 0.0;
};

struct HMaterial {
  int id;
  std::vector<int> nuclide;
  std::vector<double> atom_density;
};

struct HSource {
  int sp_type = 0;  // 0 point, 1 box
  int an_type = 0;  // 0 isotropic, 1 monodirectional
  int en_type = 0;  // 0 discrete, 1 maxwell
  int dom_type = -1;  // -1 none, 0 cell, 1 material, 2 universe
  std::vector<double> sp, en;
  double uref[3] = {1, 0, 0};
  double strength = 1.0;
  std::vector<int> dom_ids;
};

struct HWeightWindows {
  int id = -1, mesh = -1;
  std::vector<double> ebounds, lower, upper;  // lower/upper [e][m]
  double survival_ratio = 3.0, max_lb_ratio = 1.0, weight_cutoff = 1.0e-38;
  int max_split = 10;
};

struct HWWGenerator {
  int mesh = -1;
  std::vector<double> ebounds;
  int max_realizations = 1, update_interval = 1;
  bool on_the_fly = true;
  std::string method = "magic", value = "mean";
  double threshold = 1.0, ratio = 5.0;
  int tally = -1;  // index of the generated tally
  int ww = -1;     // index of the weight windows it updates
};

struct HModel {
  // output (src/settings.cpp: <output><tallies>, <output><path>)
  bool output_tallies = true;
  std::string path_output;  // directory for tallies.out (default: the input's directory)
  // settings (src/settings.cpp)
  int64_t n_particles = 0;
  int n_batches = 0, n_inactive = 0;
  int64_t seed = 1;
  uint64_t stride = 152917ULL;
  int n_log_bins = 8000;
  bool event_based = false;
  int64_t max_particles_in_flight = 0;  // 0: library chooses
  int64_t max_history_splits = 10000000;
  int max_particle_events = 1000000;
  double energy_cutoff = 0.0;
  double time_cutoff = 1.7976931348623157e308;  // neutron time cutoff in s (largest double: none)
  bool ww_on = false;
  int max_lost_particles = 10;
  double rel_max_lost_particles = 1.0e-6;
  int xs_precision = 64;  // 64 or 32 (FP32 tables)
  bool eigenvalue = false;  // run_mode eigenvalue (one generation per batch)

  std::vector<HNuclide> nuclides;
  std::vector<HMaterial> materials;
  std::vector<HSurface> surfaces;
  std::vector<HCell> cells;
  std::vector<int> univ_ids;
  std::vector<std::vector<int>> universes;
  std::vector<HLattice> lattices;
  int root_universe = 0;
  int n_coord_levels = 1;
  std::vector<HMesh> meshes;
  std::vector<HFilter> filters;
  std::vector<HTally> tallies;
  HSource source;
  std::vector<HWeightWindows> weight_windows;
  std::vector<HWWGenerator> ww_generators;

  double energy_min = 0, energy_max = 0, log_spacing = 0;
};

// Reads <path>/model.xml (or the separate XML files) and the nuclide library.
// Throws std::runtime_error with a message on invalid input.
void load_model(const std::string& path, HModel& m);

// Build derived data: create_derived, init_grid, normalized atom densities,
// tally strides, coordinate depth (src/nuclide.cpp:359-533,
// src/simulation.cpp:682-761, src/material.cpp:417-467, src/tallies/tally.cpp:503-516).
void finalize_model(HModel& m);

}  // namespace omc
