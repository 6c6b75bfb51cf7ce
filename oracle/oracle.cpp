// ORACLE — test infrastructure only; never part of the product.
//
// CPU restatement of OpenMC's continuous-energy neutron transport path
// (fixed-source and eigenvalue runs, event-based and history-based loops),
// written from the reference's behaviour with each function citing the
// reference file:line it follows.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may load
// the library built from this file, and only to check results or as the
// timed baseline.
//
// Parity pins: prn / future_seed / init_seed are checked bit-for-bit against
// the reference's own src/random_lcg.cpp compiled from source (oracle/_ref),
// and rotate_angle / maxwell_spectrum / watt_spectrum against the golden
// values in tests/cpp_unit_tests/test_math.cpp:204-276.  Transport results on
// the synthetic models are pinned only by this restatement (the reference
// needs HDF5, pugixml, fmt and xtensor, none of which exist here).
//
// Arithmetic order follows the reference expression by expression; build with
// -ffp-contract=off so that no multiply-add is fused.
//
// Deliberate, documented simplifications (identical results for the models
// this project runs):
//  * neighbour lists (src/geometry.cpp:256-282) are an ordering optimisation;
//    for non-overlapping cells the located cell is the same as an exhaustive
//    search of the universe, which is what is done here;
//  * regions with unions are evaluated in postfix form; the truth value equals
//    the reference's infix short-circuit scan (src/cell.cpp:973-1020);
//  * the hash bin int(log(E/E_min)/spacing) (src/material.cpp:833) is clamped
//    to [0, M-1]; the reference indexes grid_index[M+1], one past the table,
//    when E equals the grid maximum exactly;
//  * an elastic-only nuclide whose cutoff lands above its elastic cross
//    section by rounding (physics.cpp:709-724, probability ~1e-16) scatters
//    elastically instead of entering the inelastic branch with no reactions.

#include <algorithm>
#include <array>
#include <functional>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---------------------------------------------------------------- constants
// include/openmc/constants.h:49-54, 81-83, 90-102
constexpr double INFTY = std::numeric_limits<double>::max();
constexpr double PI = 3.141592653589793238462643383279502884L;
constexpr double TINY_BIT = 1e-8;
constexpr double FP_PRECISION = 1e-14;
constexpr double FP_REL_PRECISION = 1e-5;
constexpr double FP_COINCIDENT = 1e-12;
constexpr double MASS_NEUTRON_EV = 939.56542052e6;
constexpr double C_LIGHT = 2.99792458e10;
constexpr double N_AVOGADRO = 0.602214076;
constexpr int C_NONE = -1;
constexpr int MATERIAL_VOID = -1;
constexpr int SURFACE_NONE = 0;
constexpr double CACHE_INVALID = -1.0;
constexpr int32_t OP_LEFT_PAREN = std::numeric_limits<int32_t>::max();
constexpr int32_t OP_RIGHT_PAREN = OP_LEFT_PAREN - 1;
constexpr int32_t OP_COMPLEMENT = OP_LEFT_PAREN - 2;
constexpr int32_t OP_INTERSECTION = OP_LEFT_PAREN - 3;
constexpr int32_t OP_UNION = OP_LEFT_PAREN - 4;
constexpr int N_STREAMS = 4;
constexpr int STREAM_TRACKING = 0;
constexpr int STREAM_SOURCE = 1;
constexpr int STREAM_URR_PTABLE = 2;
constexpr int MAX_COORD = 4;
constexpr int NEUTRON = 0;

// ---------------------------------------------------------------------- RNG
// src/random_lcg.cpp:11-13, 32-44, 60-120
constexpr uint64_t prn_mult = 6364136223846793005ULL;
constexpr uint64_t prn_add = 1442695040888963407ULL;

struct RngConfig {
  int64_t master_seed = 1;
  uint64_t stride = 152917ULL;  // include/openmc/random_lcg.h:18
};

double prn(uint64_t* seed)
{
  *seed = (prn_mult * (*seed) + prn_add);
  uint64_t word =
    ((*seed >> ((*seed >> 59u) + 5u)) ^ *seed) * 12605985483714917081ull;
  uint64_t result = (word >> 43u) ^ word;
  return std::ldexp(static_cast<double>(result), -64);
}

uint64_t future_seed(uint64_t n, uint64_t seed)
{
  uint64_t g = prn_mult, c = prn_add, g_new = 1, c_new = 0;
  while (n > 0) {
    if (n & 1) {
      g_new *= g;
      c_new = c_new * g + c;
    }
    c *= (g + 1);
    g *= g;
    n >>= 1;
  }
  return g_new * seed + c_new;
}

uint64_t init_seed(const RngConfig& rc, int64_t id, int offset)
{
  return future_seed(static_cast<uint64_t>(id) * rc.stride, rc.master_seed + offset);
}

void init_particle_seeds(const RngConfig& rc, int64_t id, uint64_t* seeds)
{
  for (int i = 0; i < N_STREAMS; i++)
    seeds[i] = future_seed(static_cast<uint64_t>(id) * rc.stride, rc.master_seed + i);
}

void advance_prn_seed(int64_t n, uint64_t* seed)
{
  *seed = future_seed(static_cast<uint64_t>(n), *seed);
}

// ------------------------------------------------------------------ vectors
struct Pos {
  double x = 0, y = 0, z = 0;
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double dot(const Pos& o) const { return x * o.x + y * o.y + z * o.z; }
  double norm() const { return std::sqrt(x * x + y * y + z * z); }
};
// include/openmc/position.h:140-206, src/position.cpp (component-wise)
inline Pos operator+(Pos a, const Pos& b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline Pos operator-(Pos a, const Pos& b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
inline Pos operator*(Pos a, const Pos& b) { a.x *= b.x; a.y *= b.y; a.z *= b.z; return a; }
inline Pos operator*(double v, Pos b) { b.x *= v; b.y *= v; b.z *= v; return b; }
inline Pos operator*(Pos b, double v) { b.x *= v; b.y *= v; b.z *= v; return b; }
inline Pos operator/(Pos b, double v) { b.x /= v; b.y /= v; b.z /= v; return b; }
// include/openmc/position.h:207-213
inline Pos reflect(const Pos& u, Pos n)
{
  const double projection = n.dot(u);
  const double magnitude = n.dot(n);
  n = n * (2.0 * projection / magnitude);
  return u - n;
}

// ------------------------------------------------------- sampling functions
// src/random_dist.cpp:10-45
double uniform_distribution(double a, double b, uint64_t* seed)
{
  return a + (b - a) * prn(seed);
}

double maxwell_spectrum(double T, uint64_t* seed)
{
  double r1 = prn(seed);
  double r2 = prn(seed);
  double r3 = prn(seed);
  double c = std::cos(PI / 2. * r3);
  return -T * (std::log(r1) + std::log(r2) * c * c);
}

double watt_spectrum(double a, double b, uint64_t* seed)
{
  double w = maxwell_spectrum(a, seed);
  return w + 0.25 * a * a * b +
         uniform_distribution(-1., 1., seed) * std::sqrt(a * a * b * w);
}

// src/math_functions.cpp:763-792
Pos rotate_angle(Pos u, double mu, const double* phi, uint64_t* seed)
{
  double phi_;
  if (phi != nullptr) {
    phi_ = (*phi);
  } else {
    phi_ = 2.0 * PI * prn(seed);
  }
  double sinphi = std::sin(phi_);
  double cosphi = std::cos(phi_);
  double a = std::sqrt(std::fmax(0., 1. - mu * mu));
  double b = std::sqrt(std::fmax(0., 1. - u.z * u.z));
  if (b > 1e-10) {
    return {mu * u.x + a * (u.x * u.z * cosphi - u.y * sinphi) / b,
      mu * u.y + a * (u.y * u.z * cosphi + u.x * sinphi) / b,
      mu * u.z - a * b * cosphi};
  } else {
    b = std::sqrt(1. - u.y * u.y);
    return {mu * u.x + a * (-u.x * u.y * sinphi + u.z * cosphi) / b,
      mu * u.y + a * b * sinphi,
      mu * u.z - a * (u.y * u.z * sinphi + u.x * cosphi) / b};
  }
}

// src/distribution_multi.cpp:106-112
Pos isotropic_direction(uint64_t* seed)
{
  double phi = uniform_distribution(0., 2.0 * PI, seed);
  double mu = uniform_distribution(-1., 1., seed);
  return {mu, std::sqrt(1.0 - mu * mu) * std::cos(phi),
    std::sqrt(1.0 - mu * mu) * std::sin(phi)};
}

// include/openmc/search.h:14-20
template<class T>
int64_t lower_bound_index(const T* first, const T* last, T value)
{
  if (*first == value)
    return 0;
  return std::lower_bound(first, last, value) - first - 1;
}

// ------------------------------------------------------------------ model
struct Blob {
  std::map<std::string, std::vector<int64_t>> i;
  std::map<std::string, std::vector<double>> d;
  const std::vector<int64_t>& I(const char* k) const
  {
    auto it = i.find(k);
    if (it == i.end()) throw std::runtime_error(std::string("missing array ") + k);
    return it->second;
  }
  const std::vector<double>& D(const char* k) const
  {
    auto it = d.find(k);
    if (it == d.end()) throw std::runtime_error(std::string("missing array ") + k);
    return it->second;
  }
};

Blob parse_blob(const uint8_t* p, size_t n)
{
  Blob b;
  if (n < 12 || std::memcmp(p, "OMCFLAT1", 8) != 0) throw std::runtime_error("bad blob");
  size_t off = 8;
  uint32_t cnt;
  std::memcpy(&cnt, p + off, 4); off += 4;
  for (uint32_t k = 0; k < cnt; ++k) {
    uint8_t nl = p[off++];
    std::string name(reinterpret_cast<const char*>(p + off), nl); off += nl;
    char kind = static_cast<char>(p[off++]);
    uint64_t m;
    std::memcpy(&m, p + off, 8); off += 8;
    if (kind == 'i') {
      std::vector<int64_t> v(m);
      if (m) std::memcpy(v.data(), p + off, 8 * m);
      b.i[name] = std::move(v);
    } else {
      std::vector<double> v(m);
      if (m) std::memcpy(v.data(), p + off, 8 * m);
      b.d[name] = std::move(v);
    }
    off += 8 * m;
  }
  return b;
}

struct Nuclide {
  double awr, kT;
  std::vector<double> energy;
  std::vector<double> xs;       // [G][5] TOTAL, ABSORPTION, FISSION, NU_FISSION, PHOTON_PROD
  std::vector<double> elastic;  // reactions_[0]->xs_[0].value (MT 2)
  std::vector<int> grid_index;  // [M+1]
  // MT 18 with one prompt neutron product: yield polynomial nu_c (increasing
  // powers of E), energy spectrum 1 Maxwell (sp[0] = theta) or 2 Watt
  // (sp = a, b) with restriction energy u, isotropic emission
  bool fissionable = false;
  double nu_c[2] = {0.0, 0.0};
  int spectrum = 0;
  double sp[2] = {0.0, 0.0};
  double u = 0.0;
  // src/endf.cpp:125-134 Polynomial::operator() (Horner, increasing powers)
  double nu(double E) const
  {
    double y = 0.0;
    for (int k = 1; k >= 0; --k) y = y * E + nu_c[k];
    return y;
  }
};

struct Material {
  std::vector<int> nuclide;
  std::vector<double> atom_density;
  double atom_density_i(int i, double rho) const { return atom_density[i] * rho; }
};

struct Surface {
  int type;  // 0 x-plane 1 y-plane 2 z-plane 3 x-cyl 4 y-cyl 5 z-cyl 6 sphere
  double c[4];
  int bc;    // 0 transmission 1 vacuum 2 reflective
  int id;
};

struct Cell {
  int id, universe, fill_type, fill;  // fill_type 0 material 1 universe 2 lattice
  std::vector<int32_t> expr;
  bool simple;
  Pos translation;
};

struct Lattice {
  int n[3];
  Pos ll, pitch;
  bool is_3d;
  int outer;
  std::vector<int> universes;
  bool valid(const int* i) const
  {
    return i[0] >= 0 && i[0] < n[0] && i[1] >= 0 && i[1] < n[1] && i[2] >= 0 && i[2] < n[2];
  }
  int flat(const int* i) const { return n[0] * n[1] * i[2] + n[0] * i[1] + i[0]; }
};

struct Mesh {
  int ndim;
  int shape[3];
  double ll[3], ur[3], width[3];
};

struct Filter {
  int type;  // 0 mesh 1 energy 2 particle 3 cell 4 material
  int mesh;
  int nbins;
  std::vector<double> bins;
  std::vector<int> ids;  // cell / material indices of the bins (types 3, 4)
};

struct Tally {
  int id;
  int estimator = 0;  // 0 track length, 1 collision
  std::vector<int> filters;
  std::vector<int> strides;
  std::vector<int> scores;  // 0 flux 1 total 2 absorption
  int64_t n_filter_bins;
  std::vector<double> results;  // [bins][scores][3]  VALUE, SUM, SUM_SQ
  int n_realizations = 0;
};

struct WeightWindows {
  int mesh = -1;
  std::vector<double> energy_bounds, lower, upper;  // lower/upper [e][m]
  double survival_ratio = 3.0, max_lb_ratio = 1.0, weight_cutoff = 1.0e-38;
  int max_split = 10;
};

struct WW {  // include/openmc/weight_windows.h:58-76
  double lower_weight = -1, upper_weight = 1, max_lb_ratio = 1, survival_weight = 0.5;
  double weight_cutoff = 1.0e-38;
  int max_split = 10;
  bool is_valid() const { return lower_weight >= 0.0; }
  void scale(double f)
  {
    lower_weight *= f;
    upper_weight *= f;
    survival_weight *= f;
  }
};

// ------------------------------------------------------------- particle
struct LocalCoord {
  Pos r, u;
  int cell = C_NONE, universe = C_NONE, lattice = C_NONE;
  int lattice_index[3] = {0, 0, 0};
  void reset()  // src/particle_data.cpp:40-49
  {
    cell = C_NONE;
    universe = C_NONE;
    lattice = C_NONE;
    lattice_index[0] = lattice_index[1] = lattice_index[2] = 0;
  }
};

struct BoundaryInfo {
  double distance = INFINITY;
  int surface = SURFACE_NONE;
  int coord_level = 0;
  int lattice_translation[3] = {0, 0, 0};
};

struct MicroXS {
  double total, absorption, elastic, fission = 0.0, nu_fission = 0.0;
  int index_grid;
  double interp_factor;
  double last_E = 0.0;
};

struct SourceSite {
  Pos r, u;
  double E = 0, time = 0, wgt = 1.0;
  int surf_id = SURFACE_NONE;
  int64_t parent_id = 0;  // fission sites: the parent's id and progeny number
  int progeny_id = 0;
};

struct TraceRec {
  int32_t kind, cell, material, surface_or_nuclide, grid_hash, n_coord;
  double E, dist, wgt;
};

struct Particle {
  int64_t id = 0;
  LocalCoord coord[MAX_COORD];
  int n_coord = 1;
  int cell_last[MAX_COORD];
  int n_coord_last = 1;
  Pos r_last, u_last;
  double E = 0, E_last = 0, wgt = 1, wgt_last = 1, wgt_born = 1, wgt_ww_born = -1, ww_factor = 0;
  int n_split = 0;
  double time = 0, time_last = 0;
  int surface = SURFACE_NONE;
  int material = C_NONE, material_last = C_NONE;
  double sqrtkT = -1, sqrtkT_last = 0, density_mult = 1, density_mult_last = 1;
  int cell_born = C_NONE;
  uint64_t seeds[N_STREAMS];
  int stream = STREAM_TRACKING;
  double macro_total = 0, macro_absorption = 0;
  std::vector<MicroXS> micro;
  BoundaryInfo boundary;
  double collision_distance = 0;
  int n_event = 0, n_collision = 0;
  int event_nuclide = -1;
  std::vector<SourceSite> secondary_bank;
  double keff_tally_leakage = 0;
  double keff_tally_collision = 0, keff_tally_absorption = 0, keff_tally_tracklength = 0;
  double macro_fission = 0, macro_nu_fission = 0;
  int n_progeny = 0;
  double mu = 0;
  bool lost = false;
  // trace bookkeeping
  TraceRec* trace = nullptr;
  int trace_cap = 0, trace_n = 0;
  int32_t trace_grid = 0;

  Pos& r() { return coord[0].r; }
  Pos& u() { return coord[0].u; }
  LocalCoord& lowest() { return coord[n_coord - 1]; }
  Pos& r_local() { return coord[n_coord - 1].r; }
  Pos& u_local() { return coord[n_coord - 1].u; }
  uint64_t* current_seed() { return seeds + stream; }
  bool alive() const { return wgt != 0.0; }
  void clear()  // include/openmc/particle_data.h:288-299
  {
    for (auto& c : coord) c.reset();
    n_coord = 1;
    for (auto& c : cell_last) c = C_NONE;
    n_coord_last = 1;
  }
};

// ------------------------------------------------------------- simulation
struct Sim {
  RngConfig rng;
  int64_t n_particles = 0;
  int n_batches = 0, n_inactive = 0;
  int n_log_bins = 8000;
  int64_t max_history_splits = 10000000;
  int max_particle_events = 1000000;
  double energy_cutoff = 0.0;
  double time_cutoff = INFTY;  // neutron time cutoff (src/settings.cpp:112, 723-724)
  bool ww_on = false;
  double energy_min = 0, energy_max = INFTY, log_spacing = 0;
  std::vector<Nuclide> nuclides;
  std::vector<Material> materials;
  std::vector<Surface> surfaces;
  std::vector<Cell> cells;
  std::vector<std::vector<int>> universes;
  std::vector<Lattice> lattices;
  int root_universe = 0;
  int n_coord_levels = 1;
  std::vector<Mesh> meshes;
  std::vector<Filter> filters;
  std::vector<Tally> tallies;
  int n_collision_tallies = 0;
  WeightWindows ww;
  // source
  int sp_type, an_type, en_type, dom_type;
  std::vector<double> sp_par, en_par;
  Pos u_ref;
  double strength = 1.0;
  std::vector<int64_t> dom_ids;
  std::vector<int> mat_id, cell_id;
  double cell_sqrtkT = 0;
  // globals
  double total_weight = 0, leakage = 0;
  int64_t n_lost = 0;
  std::vector<double> leak_sum;  // per batch normalised leakage (SUM, SUM_SQ)
  double leak_s1 = 0, leak_s2 = 0;
  // eigenvalue run (src/eigenvalue.cpp, src/bank.cpp)
  bool eigenvalue = false;
  double energy_max_neutron = INFTY;  // data::energy_max[neutron]
  double keff = 1.0, keff_std = 0.0;
  double k_col = 0, k_abs = 0, k_tra = 0;  // this generation's global_tally_* sums
  std::vector<SourceSite> source_bank, fission_bank;
  int64_t fission_bank_cap = 0, n_fission_sites = 0;
  int fission_bank_full = 0;
  double keff_generation = 0.0;
  std::vector<int64_t> progeny_per_particle;
  std::vector<double> k_generation;
  double k_sum[2] = {0.0, 0.0};
  // global tallies K_COLLISION, K_ABSORPTION, K_TRACKLENGTH, LEAKAGE x (VALUE, SUM, SUM_SQ)
  double gt[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double k_col_abs = 0, k_col_tra = 0, k_abs_tra = 0;
  int n_realizations = 0;
};

// ---------------------------------------------------------- XS data setup
// src/nuclide.cpp:359-453 create_derived: reactions in MT order (2, 18,
// 102); total += xs of each; MT 18 adds to fission and absorption, MT 102
// (disappearance) to absorption; then nu_fission = nu(E) x fission per
// grid point.  fis is null for a nuclide without MT 18.
void create_derived(Nuclide& nuc, const double* el, const double* fis, const double* cap, int G)
{
  nuc.xs.assign(static_cast<size_t>(G) * 5, 0.0);
  for (int k = 0; k < G; ++k) nuc.xs[5 * k + 0] += el[k];
  if (fis) {
    for (int k = 0; k < G; ++k) {
      nuc.xs[5 * k + 0] += fis[k];
      nuc.xs[5 * k + 2] += fis[k];
      nuc.xs[5 * k + 1] += fis[k];
    }
  }
  for (int k = 0; k < G; ++k) {
    nuc.xs[5 * k + 0] += cap[k];
    nuc.xs[5 * k + 1] += cap[k];
  }
  if (fis)
    for (int k = 0; k < G; ++k) nuc.xs[5 * k + 3] = nuc.nu(nuc.energy[k]) * nuc.xs[5 * k + 2];
  nuc.elastic.assign(el, el + G);
}

// src/nuclide.cpp:502-533 init_grid; the equal-lethargy points are
// start + step*k with step = (M*spacing - 0)/M (xt::linspace)
void init_grid(Nuclide& nuc, double E_min, double E_max, int M)
{
  double spacing = std::log(E_max / E_min) / M;
  double stop = M * spacing;
  double step = stop / M;
  nuc.grid_index.assign(M + 1, 0);
  int j = 0;
  int G = static_cast<int>(nuc.energy.size());
  for (int k = 0; k <= M; ++k) {
    double umesh = 0.0 + step * k;
    if (k == M) umesh = stop;
    while (std::log(nuc.energy[j + 1] / E_min) <= umesh) {
      if (j + 2 == G) break;
      ++j;
    }
    nuc.grid_index[k] = j;
  }
}

// ---------------------------------------------------------------- surfaces
// src/surface.cpp:116-140, 207-242, 384-456, 549-570
double surf_evaluate(const Surface& s, const Pos& r)
{
  switch (s.type) {
  case 0: return r.x - s.c[0];
  case 1: return r.y - s.c[0];
  case 2: return r.z - s.c[0];
  case 3: { double a = r.y - s.c[0], b = r.z - s.c[1]; return a * a + b * b - s.c[2] * s.c[2]; }
  case 4: { double a = r.x - s.c[0], b = r.z - s.c[1]; return a * a + b * b - s.c[2] * s.c[2]; }
  case 5: { double a = r.x - s.c[0], b = r.y - s.c[1]; return a * a + b * b - s.c[2] * s.c[2]; }
  default: {
    double x = r.x - s.c[0], y = r.y - s.c[1], z = r.z - s.c[2];
    return x * x + y * y + z * z - s.c[3] * s.c[3];
  }
  }
}

double plane_distance(double r_i, double u_i, bool coincident, double offset)
{
  const double f = offset - r_i;
  if (coincident || std::abs(f) < FP_COINCIDENT || u_i == 0.0)
    return INFTY;
  const double d = f / u_i;
  if (d < 0.0)
    return INFTY;
  return d;
}

double cylinder_distance(double u1, double r2_, double u2, double r3_, double u3,
  bool coincident, double offset1, double offset2, double radius)
{
  const double a = 1.0 - u1 * u1;
  if (a == 0.0)
    return INFTY;
  const double r2 = r2_ - offset1;
  const double r3 = r3_ - offset2;
  const double k = r2 * u2 + r3 * u3;
  const double c = r2 * r2 + r3 * r3 - radius * radius;
  const double quad = k * k - a * c;
  if (quad < 0.0) {
    return INFTY;
  } else if (coincident || std::abs(c) < FP_COINCIDENT) {
    if (k >= 0.0) {
      return INFTY;
    } else {
      return (-k + std::sqrt(quad)) / a;
    }
  } else if (c < 0.0) {
    return (-k + std::sqrt(quad)) / a;
  } else {
    const double d = (-k - std::sqrt(quad)) / a;
    if (d < 0.0)
      return INFTY;
    return d;
  }
}

// src/surface.cpp SurfaceSphere::distance
double sphere_distance(const Surface& s, const Pos& r, const Pos& u, bool coincident)
{
  const double x = r.x - s.c[0];
  const double y = r.y - s.c[1];
  const double z = r.z - s.c[2];
  const double k = x * u.x + y * u.y + z * u.z;
  const double c = x * x + y * y + z * z - s.c[3] * s.c[3];
  const double quad = k * k - c;
  if (quad < 0.0) {
    return INFTY;
  } else if (coincident || std::abs(c) < FP_COINCIDENT) {
    if (k >= 0.0) {
      return INFTY;
    } else {
      return -k + std::sqrt(quad);
    }
  } else if (c < 0.0) {
    return -k + std::sqrt(quad);
  } else {
    const double d = -k - std::sqrt(quad);
    if (d < 0.0)
      return INFTY;
    return d;
  }
}

double surf_distance(const Surface& s, const Pos& r, const Pos& u, bool coincident)
{
  switch (s.type) {
  case 0: return plane_distance(r.x, u.x, coincident, s.c[0]);
  case 1: return plane_distance(r.y, u.y, coincident, s.c[0]);
  case 2: return plane_distance(r.z, u.z, coincident, s.c[0]);
  case 3: return cylinder_distance(u.x, r.y, u.y, r.z, u.z, coincident, s.c[0], s.c[1], s.c[2]);
  case 4: return cylinder_distance(u.y, r.x, u.x, r.z, u.z, coincident, s.c[0], s.c[1], s.c[2]);
  case 5: return cylinder_distance(u.z, r.x, u.x, r.y, u.y, coincident, s.c[0], s.c[1], s.c[2]);
  default: return sphere_distance(s, r, u, coincident);
  }
}

Pos surf_normal(const Surface& s, const Pos& r)
{
  switch (s.type) {
  case 0: return {1., 0., 0.};
  case 1: return {0., 1., 0.};
  case 2: return {0., 0., 1.};
  case 3: return {0.0, 2.0 * (r.y - s.c[0]), 2.0 * (r.z - s.c[1])};
  case 4: return {2.0 * (r.x - s.c[0]), 0.0, 2.0 * (r.z - s.c[1])};
  case 5: return {2.0 * (r.x - s.c[0]), 2.0 * (r.y - s.c[1]), 0.0};
  default: return {2.0 * (r.x - s.c[0]), 2.0 * (r.y - s.c[1]), 2.0 * (r.z - s.c[2])};
  }
}

bool surf_sense(const Surface& s, const Pos& r, const Pos& u)
{
  const double f = surf_evaluate(s, r);
  if (std::abs(f) < FP_COINCIDENT) {
    return u.dot(surf_normal(s, r)) > 0.0;
  }
  return f > 0.0;
}

// ------------------------------------------------------------ cell regions
// src/cell.cpp:910-936
std::pair<double, int32_t> region_distance(const Sim& S, const Cell& c, const Pos& r, const Pos& u, int32_t on_surface)
{
  double min_dist = INFTY;
  int32_t i_surf = std::numeric_limits<int32_t>::max();
  for (int32_t token : c.expr) {
    if (token >= OP_UNION)
      continue;
    bool coincident = std::abs(token) == std::abs(on_surface);
    double d = surf_distance(S.surfaces[std::abs(token) - 1], r, u, coincident);
    if (d < min_dist) {
      if (min_dist - d >= FP_PRECISION * min_dist) {
        min_dist = d;
        i_surf = -token;
      }
    }
  }
  return {min_dist, i_surf};
}

// src/cell.cpp:951-969 (simple) and postfix evaluation for complex regions
bool region_contains(const Sim& S, const Cell& c, const Pos& r, const Pos& u, int32_t on_surface)
{
  if (c.simple) {
    for (int32_t token : c.expr) {
      if (token == on_surface) {
      } else if (-token == on_surface) {
        return false;
      } else {
        bool sense = surf_sense(S.surfaces[std::abs(token) - 1], r, u);
        if (sense != (token > 0))
          return false;
      }
    }
    return true;
  }
  bool stack[64];
  int sp = 0;
  for (int32_t token : c.expr) {
    if (token < OP_UNION) {
      bool v;
      if (token == on_surface) v = true;
      else if (-token == on_surface) v = false;
      else v = (surf_sense(S.surfaces[std::abs(token) - 1], r, u) == (token > 0));
      stack[sp++] = v;
    } else if (token == OP_COMPLEMENT) {
      stack[sp - 1] = !stack[sp - 1];
    } else if (token == OP_INTERSECTION) {
      bool b = stack[--sp];
      stack[sp - 1] = stack[sp - 1] && b;
    } else if (token == OP_UNION) {
      bool b = stack[--sp];
      stack[sp - 1] = stack[sp - 1] || b;
    }
  }
  return sp > 0 ? stack[0] : true;
}

// ---------------------------------------------------------------- lattice
// src/lattice.cpp:252-361
std::pair<double, std::array<int, 3>> lattice_distance(const Lattice& lat, const Pos& r, const Pos& u)
{
  double x = r.x, y = r.y, z = r.z;
  double x0 = std::copysign(0.5 * lat.pitch.x, u.x);
  double y0 = std::copysign(0.5 * lat.pitch.y, u.y);
  double d = INFTY;
  std::array<int, 3> trans {0, 0, 0};
  if ((std::abs(x - x0) > FP_PRECISION) && u.x != 0) {
    d = (x0 - x) / u.x;
    trans = (u.x > 0) ? std::array<int, 3> {1, 0, 0} : std::array<int, 3> {-1, 0, 0};
  }
  if ((std::abs(y - y0) > FP_PRECISION) && u.y != 0) {
    double this_d = (y0 - y) / u.y;
    if (this_d < d) {
      d = this_d;
      trans = (u.y > 0) ? std::array<int, 3> {0, 1, 0} : std::array<int, 3> {0, -1, 0};
    }
  }
  if (lat.is_3d) {
    double z0 = std::copysign(0.5 * lat.pitch.z, u.z);
    if ((std::abs(z - z0) > FP_PRECISION) && u.z != 0) {
      double this_d = (z0 - z) / u.z;
      if (this_d < d) {
        d = this_d;
        trans = (u.z > 0) ? std::array<int, 3> {0, 0, 1} : std::array<int, 3> {0, 0, -1};
      }
    }
  }
  return {d, trans};
}

void lattice_get_indices(const Lattice& lat, const Pos& r, const Pos& u, int* result)
{
  double ix_ = (r.x - lat.ll.x) / lat.pitch.x;
  long ix_close = std::lround(ix_);
  if (std::abs(ix_ - ix_close) < FP_COINCIDENT) {
    result[0] = (u.x > 0) ? ix_close : ix_close - 1;
  } else {
    result[0] = std::floor(ix_);
  }
  double iy_ = (r.y - lat.ll.y) / lat.pitch.y;
  long iy_close = std::lround(iy_);
  if (std::abs(iy_ - iy_close) < FP_COINCIDENT) {
    result[1] = (u.y > 0) ? iy_close : iy_close - 1;
  } else {
    result[1] = std::floor(iy_);
  }
  result[2] = 0;
  if (lat.is_3d) {
    double iz_ = (r.z - lat.ll.z) / lat.pitch.z;
    long iz_close = std::lround(iz_);
    if (std::abs(iz_ - iz_close) < FP_COINCIDENT) {
      result[2] = (u.z > 0) ? iz_close : iz_close - 1;
    } else {
      result[2] = std::floor(iz_);
    }
  }
}

Pos lattice_local_position(const Lattice& lat, Pos r, const int* i)
{
  r.x -= (lat.ll.x + (i[0] + 0.5) * lat.pitch.x);
  r.y -= (lat.ll.y + (i[1] + 0.5) * lat.pitch.y);
  if (lat.is_3d) {
    r.z -= (lat.ll.z + (i[2] + 0.5) * lat.pitch.z);
  }
  return r;
}

// --------------------------------------------------------------- find cell
void mark_as_lost(Sim& S, Particle& p)
{
  p.wgt = 0.0;
  p.lost = true;
#pragma omp atomic
  S.n_lost += 1;
}

// src/universe.cpp:40-59
bool universe_find_cell(const Sim& S, Particle& p)
{
  int i_univ = p.lowest().universe;
  for (int i_cell : S.universes[i_univ]) {
    if (S.cells[i_cell].universe != i_univ)
      continue;
    if (region_contains(S, S.cells[i_cell], p.r_local(), p.u_local(), p.surface)) {
      p.lowest().cell = i_cell;
      return true;
    }
  }
  return false;
}

// src/geometry.cpp:102-252 (neighbour-list branch folded into the exhaustive search)
bool find_cell_inner(Sim& S, Particle& p)
{
  bool found = false;
  for (;; ++p.n_coord) {
    found = universe_find_cell(S, p);
    if (!found)
      return found;
    int i_cell = p.lowest().cell;
    const Cell& c = S.cells[i_cell];
    if (c.fill_type == 0) {
      p.material_last = p.material;
      p.material = c.fill;
      p.sqrtkT_last = p.sqrtkT;
      p.sqrtkT = S.cell_sqrtkT;
      p.density_mult_last = p.density_mult;
      p.density_mult = 1.0;
      return true;
    } else if (c.fill_type == 1) {
      LocalCoord& coord = p.coord[p.n_coord];
      coord.universe = c.fill;
      coord.r = p.r_local();
      coord.u = p.u_local();
      coord.r = coord.r - c.translation;
    } else {
      const Lattice& lat = S.lattices[c.fill];
      LocalCoord& coord = p.coord[p.n_coord];
      coord.r = p.r_local();
      coord.u = p.u_local();
      coord.r = coord.r - c.translation;
      lattice_get_indices(lat, coord.r, coord.u, coord.lattice_index);
      coord.r = lattice_local_position(lat, coord.r, coord.lattice_index);
      coord.lattice = c.fill;
      if (lat.valid(coord.lattice_index)) {
        coord.universe = lat.universes[lat.flat(coord.lattice_index)];
      } else {
        if (lat.outer != -1) {
          coord.universe = lat.outer;
        } else {
          mark_as_lost(S, p);
          return false;
        }
      }
    }
  }
}

// src/geometry.cpp:284-298
bool exhaustive_find_cell(Sim& S, Particle& p)
{
  int i_universe = p.lowest().universe;
  if (i_universe == C_NONE) {
    p.coord[0].universe = S.root_universe;
    p.n_coord = 1;
  }
  for (int i = p.n_coord; i < S.n_coord_levels; i++)
    p.coord[i].reset();
  return find_cell_inner(S, p);
}

// src/geometry.cpp:256-282
bool neighbor_list_find_cell(Sim& S, Particle& p)
{
  for (int i = p.n_coord; i < S.n_coord_levels; i++)
    p.coord[i].reset();
  return find_cell_inner(S, p);
}

// src/geometry.cpp:301-357
void cross_lattice(Sim& S, Particle& p, const BoundaryInfo& boundary)
{
  LocalCoord& coord = p.lowest();
  const Lattice& lat = S.lattices[coord.lattice];
  coord.lattice_index[0] += boundary.lattice_translation[0];
  coord.lattice_index[1] += boundary.lattice_translation[1];
  coord.lattice_index[2] += boundary.lattice_translation[2];
  const LocalCoord& upper = p.coord[p.n_coord - 2];
  const Cell& cell = S.cells[upper.cell];
  Pos r = upper.r - cell.translation;
  p.r_local() = lattice_local_position(lat, r, coord.lattice_index);
  if (!lat.valid(coord.lattice_index)) {
    p.n_coord = 1;
    if (!exhaustive_find_cell(S, p))
      mark_as_lost(S, p);
  } else {
    p.lowest().universe = lat.universes[lat.flat(coord.lattice_index)];
    bool found = exhaustive_find_cell(S, p);
    if (!found) {
      p.n_coord = 1;
      if (!exhaustive_find_cell(S, p))
        mark_as_lost(S, p);
    }
  }
}

// src/geometry.cpp:361-453
BoundaryInfo distance_to_boundary(Sim& S, Particle& p)
{
  BoundaryInfo info;
  double d_lat = INFINITY;
  double d_surf = INFINITY;
  int32_t level_surf_cross;
  std::array<int, 3> level_lat_trans {0, 0, 0};
  for (int i = 0; i < p.n_coord; i++) {
    const LocalCoord& coord = p.coord[i];
    const Pos& r = coord.r;
    const Pos& u = coord.u;
    const Cell& c = S.cells[coord.cell];
    auto sd = region_distance(S, c, r, u, p.surface);
    d_surf = sd.first;
    level_surf_cross = sd.second;
    if (coord.lattice != C_NONE) {
      const Lattice& lat = S.lattices[coord.lattice];
      auto ld = lattice_distance(lat, r, u);
      d_lat = ld.first;
      level_lat_trans = ld.second;
      if (d_lat < 0)
        mark_as_lost(S, p);
    }
    double& d = info.distance;
    if (d_surf < d_lat - FP_COINCIDENT) {
      if (d == INFINITY || (d - d_surf) / d >= FP_REL_PRECISION) {
        d = d_surf;
        if (c.simple || d == INFTY) {
          info.surface = level_surf_cross;
        } else {
          Pos r_hit = r + d_surf * u;
          const Surface& surf = S.surfaces[std::abs(level_surf_cross) - 1];
          Pos norm = surf_normal(surf, r_hit);
          if (u.dot(norm) > 0) {
            info.surface = std::abs(level_surf_cross);
          } else {
            info.surface = -std::abs(level_surf_cross);
          }
        }
        info.lattice_translation[0] = 0;
        info.lattice_translation[1] = 0;
        info.lattice_translation[2] = 0;
        info.coord_level = i + 1;
      }
    } else {
      if (d == INFINITY || (d - d_lat) / d >= FP_REL_PRECISION) {
        d = d_lat;
        info.surface = SURFACE_NONE;
        info.lattice_translation[0] = level_lat_trans[0];
        info.lattice_translation[1] = level_lat_trans[1];
        info.lattice_translation[2] = level_lat_trans[2];
        info.coord_level = i + 1;
      }
    }
  }
  return info;
}

// ---------------------------------------------------------- cross sections
// src/nuclide.cpp:616-839 (single temperature, no URR/S(a,b)/multipole)
void nuclide_calculate_xs(const Sim& S, int i_nuc, int i_log_union, Particle& p)
{
  const Nuclide& nuc = S.nuclides[i_nuc];
  MicroXS& micro = p.micro[i_nuc];
  micro.elastic = CACHE_INVALID;
  const auto& E = nuc.energy;
  int G = static_cast<int>(E.size());
  int i_grid;
  if (p.E < E.front()) {
    i_grid = 0;
  } else if (p.E > E.back()) {
    i_grid = G - 2;
  } else {
    int i_low = nuc.grid_index[i_log_union];
    int i_high = nuc.grid_index[i_log_union + 1] + 1;
    i_grid = i_low + static_cast<int>(lower_bound_index(&E[i_low], &E[i_high], p.E));
  }
  if (E[i_grid] == E[i_grid + 1])
    ++i_grid;
  double f = (p.E - E[i_grid]) / (E[i_grid + 1] - E[i_grid]);
  micro.index_grid = i_grid;
  micro.interp_factor = f;
  micro.total = (1.0 - f) * nuc.xs[5 * i_grid + 0] + f * nuc.xs[5 * (i_grid + 1) + 0];
  micro.absorption = (1.0 - f) * nuc.xs[5 * i_grid + 1] + f * nuc.xs[5 * (i_grid + 1) + 1];
  if (nuc.fissionable) {
    micro.fission = (1.0 - f) * nuc.xs[5 * i_grid + 2] + f * nuc.xs[5 * (i_grid + 1) + 2];
    micro.nu_fission = (1.0 - f) * nuc.xs[5 * i_grid + 3] + f * nuc.xs[5 * (i_grid + 1) + 3];
  } else {
    micro.fission = 0.0;
    micro.nu_fission = 0.0;
  }
  micro.last_E = p.E;
}

// src/particle.cpp:859-870 update_neutron_xs
void update_neutron_xs(const Sim& S, int i_nuc, int i_grid, Particle& p)
{
  MicroXS& micro = p.micro[i_nuc];
  if (p.E != micro.last_E) {
    nuclide_calculate_xs(S, i_nuc, i_grid, p);
  }
}

// src/material.cpp:829-901
void material_calculate_xs(Sim& S, Particle& p)
{
  p.macro_total = 0.0;
  p.macro_absorption = 0.0;
  p.macro_fission = 0.0;
  p.macro_nu_fission = 0.0;
  const Material& mat = S.materials[p.material];
  int i_grid = std::log(p.E / S.energy_min) / S.log_spacing;
  i_grid = std::min(std::max(i_grid, 0), S.n_log_bins - 1);
  uint32_t h = 0;
  for (size_t i = 0; i < mat.nuclide.size(); ++i) {
    int i_nuclide = mat.nuclide[i];
    update_neutron_xs(S, i_nuclide, i_grid, p);
    const MicroXS& micro = p.micro[i_nuclide];
    h = h * 31u + static_cast<uint32_t>(micro.index_grid);
    double atom_density = mat.atom_density_i(static_cast<int>(i), p.density_mult);
    p.macro_total += atom_density * micro.total;
    p.macro_absorption += atom_density * micro.absorption;
    p.macro_fission += atom_density * micro.fission;
    p.macro_nu_fission += atom_density * micro.nu_fission;
  }
  p.trace_grid = static_cast<int32_t>(h);
}

// src/nuclide.cpp:578-590
void calculate_elastic_xs(const Sim& S, int i_nuc, Particle& p)
{
  MicroXS& micro = p.micro[i_nuc];
  int i_grid = micro.index_grid;
  double f = micro.interp_factor;
  const auto& xs = S.nuclides[i_nuc].elastic;
  micro.elastic = (1.0 - f) * xs[i_grid] + f * xs[i_grid + 1];
}

// ------------------------------------------------------------------ tallies
// src/mesh.cpp:1328-1369 RegularMesh helpers
int mesh_index_in_direction(const Mesh& m, double r, int i)
{
  return static_cast<int>(std::ceil((r - m.ll[i]) / m.width[i]));
}

struct MeshDistance {
  int next_index = -1;
  bool max_surface = true;
  double distance = INFTY;
};

MeshDistance mesh_distance_to_grid_boundary(const Mesh& m, const int* ijk, int i, const Pos& r0, const Pos& u)
{
  MeshDistance d;
  d.next_index = ijk[i];
  if (std::abs(u[i]) < FP_PRECISION)
    return d;
  d.max_surface = (u[i] > 0);
  if (d.max_surface && (ijk[i] <= m.shape[i])) {
    d.next_index++;
    d.distance = ((m.ll[i] + ijk[i] * m.width[i]) - r0[i]) / u[i];
  } else if (!d.max_surface && (ijk[i] >= 1)) {
    d.next_index--;
    d.distance = ((m.ll[i] + (ijk[i] - 1) * m.width[i]) - r0[i]) / u[i];
  }
  return d;
}

// src/mesh.cpp:874-886
void mesh_get_indices(const Mesh& m, const Pos& r, int* ijk, bool& in_mesh)
{
  in_mesh = true;
  for (int i = 0; i < m.ndim; ++i) {
    ijk[i] = mesh_index_in_direction(m, r[i], i);
    if (ijk[i] < 1 || ijk[i] > m.shape[i])
      in_mesh = false;
  }
}

int mesh_bin_from_indices(const Mesh& m, const int* ijk)
{
  switch (m.ndim) {
  case 1: return ijk[0] - 1;
  case 2: return (ijk[1] - 1) * m.shape[0] + ijk[0] - 1;
  default: return ((ijk[2] - 1) * m.shape[1] + (ijk[1] - 1)) * m.shape[0] + ijk[0] - 1;
  }
}

// src/mesh.cpp:999-1146 raytrace_mesh + bins_crossed
void mesh_bins_crossed(const Mesh& m, const Pos& r0, const Pos& r1, const Pos& u,
  std::vector<int>& bins, std::vector<double>& lengths)
{
  double total_distance = (r1 - r0).norm();
  if (total_distance == 0.0)
    return;
  const Pos& global_r = r0;
  const Pos& local_r = r0;
  const int n = m.ndim;
  bool in_mesh;
  double traveled_distance = 0.0;
  int ijk[3] = {0, 0, 0};
  mesh_get_indices(m, global_r + TINY_BIT * u, ijk, in_mesh);
  if (total_distance < 2 * TINY_BIT) {
    if (in_mesh) {
      bins.push_back(mesh_bin_from_indices(m, ijk));
      lengths.push_back(1.0);
    }
    return;
  }
  MeshDistance distances[3];
  for (int k = 0; k < n; ++k)
    distances[k] = mesh_distance_to_grid_boundary(m, ijk, k, local_r, u);
  while (true) {
    if (in_mesh) {
      int k = 0;
      for (int kk = 1; kk < 3; ++kk)
        if (distances[kk].distance < distances[k].distance) k = kk;
      bins.push_back(mesh_bin_from_indices(m, ijk));
      lengths.push_back((std::min(distances[k].distance, total_distance) - traveled_distance) / total_distance);
      traveled_distance = distances[k].distance;
      if (traveled_distance >= total_distance)
        return;
      ijk[k] = distances[k].next_index;
      distances[k] = mesh_distance_to_grid_boundary(m, ijk, k, local_r, u);
      in_mesh = ((ijk[k] >= 1) && (ijk[k] <= m.shape[k]));
    } else {
      int k_max = -1;
      for (int k = 0; k < n; ++k) {
        if ((ijk[k] < 1 || ijk[k] > m.shape[k]) && (distances[k].distance > traveled_distance)) {
          traveled_distance = distances[k].distance;
          k_max = k;
        }
      }
      if (k_max == -1) {
        traveled_distance += TINY_BIT;
      }
      if (traveled_distance >= total_distance)
        return;
      mesh_get_indices(m, global_r + (traveled_distance + TINY_BIT) * u, ijk, in_mesh);
      for (int k = 0; k < n; ++k)
        distances[k] = mesh_distance_to_grid_boundary(m, ijk, k, local_r, u);
    }
  }
}

// src/tallies/tally_scoring.cpp:2416-2541 with FilterBinIter :31-139 and
// score_general_ce_nonanalog :578-1106 (flux, total, absorption scores)
// Bins of a cell filter (src/tallies/filter_cell.cpp:48-58: every coordinate
// level whose cell is in the filter) and of a material filter
// (src/tallies/filter_material.cpp:47-55).
void cell_material_bins(const Filter& F, const Particle& p, std::vector<int>& bins, std::vector<double>& w)
{
  if (F.type == 3) {
    for (int i = 0; i < p.n_coord; ++i)
      for (size_t b = 0; b < F.ids.size(); ++b)
        if (F.ids[b] == p.coord[i].cell) {
          bins.push_back(static_cast<int>(b));
          w.push_back(1.0);
        }
  } else {
    for (size_t b = 0; b < F.ids.size(); ++b)
      if (F.ids[b] == p.material) {
        bins.push_back(static_cast<int>(b));
        w.push_back(1.0);
      }
  }
}

// Adds score x weight for every combination of the tally's filter bins
// (src/tallies/tally_scoring.cpp:31-139 FilterBinIter, last filter fastest).
void score_bins(Tally& tally, const std::vector<std::vector<int>>& fbins,
  const std::vector<std::vector<double>>& fw, double flux, const Particle& p)
{
  int nf = static_cast<int>(tally.filters.size());
  std::vector<int> ib(nf, 0);
  int ns = static_cast<int>(tally.scores.size());
  while (true) {
    int64_t index = 0;
    double weight = 1.;
    for (int i = 0; i < nf; ++i) {
      int f = tally.filters[i];
      index += static_cast<int64_t>(fbins[f][ib[i]]) * tally.strides[i];
      weight *= fw[f][ib[i]];
    }
    for (int s = 0; s < ns; ++s) {
      double score;
      switch (tally.scores[s]) {
      case 0: score = flux; break;
      case 1: score = p.macro_total * flux; break;
      default: score = p.macro_absorption * flux; break;
      }
      double* slot = &tally.results[(index * ns + s) * 3];
#pragma omp atomic
      *slot += score * weight;
    }
    int i = nf - 1;
    for (; i >= 0; --i) {
      int f = tally.filters[i];
      if (ib[i] < static_cast<int>(fbins[f].size()) - 1) {
        ++ib[i];
        break;
      } else {
        ib[i] = 0;
      }
    }
    if (i < 0) break;
  }
}

// src/tallies/tally_scoring.cpp:2543-2600 score_collision_tally: after the
// collision, flux = wgt_last / Sigma_t with the pre-collision macroscopic
// cross sections; mesh filters bin the collision site, energy filters the
// pre-collision energy.
void score_collision_tally(Sim& S, Particle& p)
{
  const double flux = p.wgt_last / p.macro_total;
  std::vector<std::vector<int>> fbins(S.filters.size());
  std::vector<std::vector<double>> fw(S.filters.size());
  for (auto& tally : S.tallies) {
    if (tally.estimator != 1) continue;
    bool empty = false;
    for (int f : tally.filters) {
      fbins[f].clear();
      fw[f].clear();
      const Filter& F = S.filters[f];
      if (F.type == 0) {
        int ijk[3];
        bool in_mesh;
        mesh_get_indices(S.meshes[F.mesh], p.r(), ijk, in_mesh);
        if (in_mesh) {
          fbins[f].push_back(mesh_bin_from_indices(S.meshes[F.mesh], ijk));
          fw[f].push_back(1.0);
        }
      } else if (F.type == 1) {
        double E = p.E_last;
        if (E >= F.bins.front() && E <= F.bins.back()) {
          fbins[f].push_back(static_cast<int>(lower_bound_index(F.bins.data(), F.bins.data() + F.bins.size(), E)));
          fw[f].push_back(1.0);
        }
      } else if (F.type == 2) {
        fbins[f].push_back(0);
        fw[f].push_back(1.0);
      } else {
        cell_material_bins(F, p, fbins[f], fw[f]);
      }
      if (fbins[f].empty()) empty = true;
    }
    if (!empty) score_bins(tally, fbins, fw, flux, p);
  }
}

void score_tracklength_tally(Sim& S, Particle& p, double distance)
{
  double flux = p.wgt * distance;
  std::vector<std::vector<int>> fbins(S.filters.size());
  std::vector<std::vector<double>> fw(S.filters.size());
  std::vector<bool> present(S.filters.size(), false);
  for (auto& tally : S.tallies) {
    if (tally.estimator != 0) continue;
    bool empty = false;
    for (int f : tally.filters) {
      if (!present[f]) {
        const Filter& F = S.filters[f];
        if (F.type == 0) {
          mesh_bins_crossed(S.meshes[F.mesh], p.r_last, p.r(), p.u(), fbins[f], fw[f]);
        } else if (F.type == 3 || F.type == 4) {
          cell_material_bins(F, p, fbins[f], fw[f]);
        } else if (F.type == 1) {
          double E = p.E_last;
          if (E >= F.bins.front() && E <= F.bins.back()) {
            fbins[f].push_back(static_cast<int>(lower_bound_index(F.bins.data(), F.bins.data() + F.bins.size(), E)));
            fw[f].push_back(1.0);
          }
        } else {
          fbins[f].push_back(0);
          fw[f].push_back(1.0);
        }
        present[f] = true;
      }
      if (fbins[f].empty()) empty = true;
    }
    if (empty)
      continue;
    score_bins(tally, fbins, fw, flux, p);
  }
}

// --------------------------------------------------------- weight windows
// src/weight_windows.cpp:375-411
WW get_weight_window(const Sim& S, Particle& p)
{
  const Mesh& m = S.meshes[S.ww.mesh];
  int ijk[3];
  bool in_mesh;
  mesh_get_indices(m, p.r(), ijk, in_mesh);
  if (!in_mesh)
    return {};
  double E = p.E;
  const auto& eb = S.ww.energy_bounds;
  if (E < eb.front() || E > eb.back())
    return {};
  int energy_bin = static_cast<int>(lower_bound_index(eb.data(), eb.data() + eb.size(), E));
  int mesh_bin = mesh_bin_from_indices(m, ijk);
  int64_t n_mesh = static_cast<int64_t>(m.shape[0]) * m.shape[1] * m.shape[2];
  WW ww;
  ww.lower_weight = S.ww.lower[energy_bin * n_mesh + mesh_bin];
  ww.upper_weight = S.ww.upper[energy_bin * n_mesh + mesh_bin];
  ww.survival_weight = ww.lower_weight * S.ww.survival_ratio;
  ww.max_lb_ratio = S.ww.max_lb_ratio;
  ww.max_split = S.ww.max_split;
  ww.weight_cutoff = S.ww.weight_cutoff;
  return ww;
}

// src/physics_common.cpp:12-19
void russian_roulette(Particle& p, double weight_survive)
{
  if (weight_survive * prn(p.current_seed()) < p.wgt) {
    p.wgt = weight_survive;
  } else {
    p.wgt = 0.;
  }
}

// src/particle.cpp:95-112
void split(Particle& p, double wgt)
{
  SourceSite s;
  s.wgt = wgt;
  s.r = p.r();
  s.u = p.u();
  s.E = p.E;
  s.time = p.time;
  s.surf_id = p.surface;
  p.secondary_bank.push_back(s);
}

// src/weight_windows.cpp:56-146
void apply_weight_windows(Sim& S, Particle& p)
{
  if (!S.ww_on)
    return;
  if (p.E <= 0 || !p.alive())
    return;
  WW weight_window = get_weight_window(S, p);
  if (p.wgt_ww_born == -1.0) {
    if (weight_window.is_valid()) {
      p.wgt_ww_born = (weight_window.lower_weight + weight_window.upper_weight) / 2;
    } else {
      p.wgt_ww_born = 1.0;
    }
  }
  if (!weight_window.is_valid())
    return;
  weight_window.scale(p.wgt_born / p.wgt_ww_born);
  double weight = p.wgt;
  if (p.wgt < weight_window.weight_cutoff) {
    p.wgt = 0.0;
    return;
  }
  if (p.ww_factor == 0.0 && weight_window.max_lb_ratio > 1.0 &&
      p.wgt > weight_window.lower_weight * weight_window.max_lb_ratio) {
    p.ww_factor = p.wgt / (weight_window.lower_weight * weight_window.max_lb_ratio);
  }
  if (p.ww_factor > 1.0)
    weight_window.scale(p.ww_factor);
  if (weight > weight_window.upper_weight) {
    if (p.n_split >= S.max_history_splits)
      return;
    double n_split = std::ceil(weight / weight_window.upper_weight);
    double max_split = weight_window.max_split;
    n_split = std::min(n_split, max_split);
    p.n_split += n_split;
    int i_split = std::round(n_split);
    for (int l = 0; l < i_split - 1; l++) {
      split(p, weight / n_split);
    }
    p.wgt = weight / n_split;
  } else if (weight <= weight_window.lower_weight) {
    double weight_survive = std::min(weight * weight_window.max_split, weight_window.survival_weight);
    russian_roulette(p, weight_survive);
  }
}

// ----------------------------------------------------------------- physics
// src/physics.cpp:990-1041
Pos sample_cxs_target_velocity(double awr, double E, Pos u, double kT, uint64_t* seed)
{
  double beta_vn = std::sqrt(awr * E / kT);
  double alpha = 1.0 / (1.0 + std::sqrt(PI) * beta_vn / 2.0);
  double beta_vt_sq;
  double mu;
  while (true) {
    double r1 = prn(seed);
    double r2 = prn(seed);
    if (prn(seed) < alpha) {
      beta_vt_sq = -std::log(r1 * r2);
    } else {
      double c = std::cos(PI / 2.0 * prn(seed));
      beta_vt_sq = -std::log(r1) - std::log(r2) * c * c;
    }
    double beta_vt = std::sqrt(beta_vt_sq);
    mu = uniform_distribution(-1., 1., seed);
    double accept_prob =
      std::sqrt(beta_vn * beta_vn + beta_vt_sq - 2 * beta_vn * beta_vt * mu) / (beta_vn + beta_vt);
    if (prn(seed) < accept_prob)
      break;
  }
  double vt = std::sqrt(beta_vt_sq * kT / awr);
  return vt * rotate_angle(u, mu, nullptr, seed);
}

// src/physics.cpp:836-874 (non-resonant nuclides)
Pos sample_target_velocity(const Nuclide& nuc, double E, Pos u, double kT, uint64_t* seed)
{
  if (E >= 400.0 * kT && nuc.awr > 1.0)
    return {};
  return sample_cxs_target_velocity(nuc.awr, E, u, kT, seed);
}

// src/physics.cpp:754-818
void elastic_scatter(Sim& S, int i_nuclide, double kT, Particle& p)
{
  const Nuclide& nuc = S.nuclides[i_nuclide];
  double vel = std::sqrt(p.E);
  double awr = nuc.awr;
  Pos v_n = vel * p.u();
  Pos v_t = sample_target_velocity(nuc, p.E, p.u(), kT, p.current_seed());
  Pos v_cm = (v_n + awr * v_t) / (awr + 1.0);
  v_n = v_n - v_cm;
  vel = v_n.norm();
  double mu_cm = uniform_distribution(-1., 1., p.current_seed());
  Pos u_cm = v_n / vel;
  v_n = vel * rotate_angle(u_cm, mu_cm, nullptr, p.current_seed());
  v_n = v_n + v_cm;
  p.E = v_n.dot(v_n);
  vel = std::sqrt(p.E);
  p.mu = p.u().dot(v_n) / vel;
  p.u() = v_n / vel;
  if (std::abs(p.mu) > 1.0)
    p.mu = std::copysign(1.0, p.mu);
}

// src/physics.cpp:674-752 (elastic only)
void scatter(Sim& S, Particle& p, int i_nuclide)
{
  MicroXS& micro = p.micro[i_nuclide];
  double cutoff = prn(p.current_seed()) * (micro.total - micro.absorption);
  if (micro.elastic == CACHE_INVALID)
    calculate_elastic_xs(S, i_nuclide, p);
  double prob = micro.elastic - 0.0;
  (void)cutoff;
  (void)prob;
  // elastic branch (prob > cutoff) and the measure-zero fall-through both
  // perform elastic scattering for MT2/MT102-only nuclides
  double kT = S.nuclides[i_nuclide].kT;
  elastic_scatter(S, i_nuclide, kT, p);
}

// src/physics.cpp:494-518
int sample_nuclide(Sim& S, Particle& p)
{
  double cutoff = prn(p.current_seed()) * p.macro_total;
  const Material& mat = S.materials[p.material];
  int n = static_cast<int>(mat.nuclide.size());
  double prob = 0.0;
  for (int i = 0; i < n; ++i) {
    int i_nuclide = mat.nuclide[i];
    double atom_density = mat.atom_density_i(i, p.density_mult);
    prob += atom_density * p.micro[i_nuclide].total;
    if (prob >= cutoff)
      return i_nuclide;
  }
  throw std::runtime_error("Did not sample any nuclide during collision.");
}

// src/physics.cpp:638-672 (analog): the absorption estimate of k-effective
// is scored when the disappearance happens
void absorption(Sim& S, Particle& p, int i_nuclide)
{
  if (p.micro[i_nuclide].absorption > prn(p.current_seed()) * p.micro[i_nuclide].total) {
    if (S.eigenvalue)
      p.keff_tally_absorption += p.wgt * p.micro[i_nuclide].nu_fission / p.micro[i_nuclide].absorption;
    p.wgt = 0.0;
  }
}

// src/physics.cpp:1043-1115 sample_fission_neutron for a prompt-only MT 18
// (nu_d = 0: the delayed test draws one number and never passes) whose
// neutron product is an uncorrelated isotropic angle (mu uniform in [-1, 1],
// src/secondary_uncorrelated.cpp) and a Maxwell or Watt spectrum with
// restriction energy (src/distribution_energy.cpp:282-360); energies at or
// above the data's maximum are resampled.
void sample_fission_neutron(const Sim& S, int i_nuclide, SourceSite& site, Particle& p)
{
  const Nuclide& nuc = S.nuclides[i_nuclide];
  double E_in = p.E;
  uint64_t* seed = p.current_seed();
  double nu_t = nuc.nu(E_in);
  double nu_d = 0.0;
  double beta = nu_d / nu_t;
  if (prn(seed) < beta)
    throw std::runtime_error("delayed neutrons are not supported");
  double mu = 0.0;
  for (int n_sample = 0;; ++n_sample) {
    mu = uniform_distribution(-1., 1., seed);
    double E_out;
    while (true) {
      E_out = nuc.spectrum == 1 ? maxwell_spectrum(nuc.sp[0], seed) : watt_spectrum(nuc.sp[0], nuc.sp[1], seed);
      if (E_out <= E_in - nuc.u) break;
    }
    site.E = E_out;
    if (site.E < S.energy_max_neutron) break;
    if (n_sample + 1 == 10000) throw std::runtime_error("Resampled energy distribution maximum number of times");
  }
  site.u = rotate_angle(p.u(), mu, nullptr, seed);
}

// src/physics.cpp:170-285 create_fission_sites (eigenvalue run, no uniform
// fission source): nu_t = wgt / keff x nu_fission / total of the sampled
// nuclide; the sites go to the shared fission bank with (parent id, progeny
// number) for the sort that makes the bank order independent of threads
void create_fission_sites(Sim& S, Particle& p, int i_nuclide)
{
  double weight = 1.0;
  const MicroXS& micro = p.micro[i_nuclide];
  double nu_t = p.wgt / S.keff * weight * micro.nu_fission / micro.total;
  int nu = static_cast<int>(nu_t);
  if (prn(p.current_seed()) <= (nu_t - nu))
    ++nu;
  if (nu == 0)
    return;
  for (int n_sites = 0; n_sites < nu; n_sites++) {
    SourceSite site;
    site.r = p.r();
    site.time = p.time;
    site.wgt = 1. / weight;
    site.surf_id = 0;
    sample_fission_neutron(S, i_nuclide, site, p);
    site.parent_id = p.id;
    site.progeny_id = p.n_progeny++;
    int64_t idx;
#pragma omp atomic capture
    idx = S.n_fission_sites++;
    if (idx >= S.fission_bank_cap) {
      // the reference warns and stops banking this particle's sites
      p.n_progeny--;
#pragma omp atomic write
      S.fission_bank_full = 1;
      break;
    }
    S.fission_bank[idx] = site;
  }
}

// src/physics.cpp:93-168
void sample_neutron_reaction(Sim& S, Particle& p)
{
  int i_nuclide = sample_nuclide(S, p);
  p.event_nuclide = i_nuclide;
  // sample_fission (src/physics.cpp:552-562) returns the only fission
  // reaction without drawing a number
  if (S.nuclides[i_nuclide].fissionable && p.micro[i_nuclide].fission > 0.0) {
    if (S.eigenvalue) create_fission_sites(S, p, i_nuclide);
  }
  if (p.micro[i_nuclide].absorption > 0.0)
    absorption(S, p, i_nuclide);
  if (!p.alive())
    return;
  scatter(S, p, i_nuclide);
  if (p.E != p.E_last)
    advance_prn_seed(static_cast<int64_t>(S.nuclides.size()), &p.seeds[STREAM_URR_PTABLE]);
}

// src/physics.cpp:43-91
void collision(Sim& S, Particle& p)
{
  ++p.n_collision;
  sample_neutron_reaction(S, p);
  apply_weight_windows(S, p);
  if (p.E < S.energy_cutoff)
    p.wgt = 0.0;
}

// ------------------------------------------------------------------ events
void trace_push(Particle& p, int kind, int sn, double dist)
{
  if (!p.trace || p.trace_n >= p.trace_cap) {
    if (p.trace) p.trace_n++;
    return;
  }
  TraceRec& t = p.trace[p.trace_n++];
  t.kind = kind;
  t.surface_or_nuclide = sn;
  t.dist = dist;
  t.wgt = p.wgt;
}

// src/particle.cpp:160-230
void event_calculate_xs(Sim& S, Particle& p)
{
  p.stream = STREAM_TRACKING;
  p.wgt_last = p.wgt;
  p.E_last = p.E;
  p.u_last = p.u();
  p.r_last = p.r();
  p.time_last = p.time;
  p.event_nuclide = -1;
  if (p.lowest().cell == C_NONE) {
    if (!exhaustive_find_cell(S, p)) {
      mark_as_lost(S, p);
      return;
    }
    if (p.cell_born == C_NONE)
      p.cell_born = p.lowest().cell;
    for (int j = 0; j < p.n_coord; ++j)
      p.cell_last[j] = p.coord[j].cell;
    p.n_coord_last = p.n_coord;
  }
  if (p.material != MATERIAL_VOID) {
    if (p.material != p.material_last || p.sqrtkT != p.sqrtkT_last ||
        p.density_mult != p.density_mult_last) {
      material_calculate_xs(S, p);
    }
  } else {
    p.macro_total = 0.0;
    p.macro_absorption = 0.0;
    p.macro_fission = 0.0;
    p.macro_nu_fission = 0.0;
    p.trace_grid = -1;
  }
  if (p.trace && p.trace_n < p.trace_cap) {
    TraceRec& t = p.trace[p.trace_n];
    t.cell = p.lowest().cell;
    t.material = p.material;
    t.grid_hash = p.trace_grid;
    t.n_coord = p.n_coord;
    t.E = p.E;
  }
}

double particle_speed(const Particle& p)  // src/particle.cpp:46-73
{
  double mass = MASS_NEUTRON_EV;
  return C_LIGHT * std::sqrt(p.E * (p.E + 2 * mass)) / (p.E + mass);
}

// src/particle.cpp:232-286
void event_advance(Sim& S, Particle& p)
{
  p.boundary = distance_to_boundary(S, p);
  if (p.macro_total == 0.0) {
    p.collision_distance = INFINITY;
  } else {
    p.collision_distance = -std::log(prn(p.current_seed())) / p.macro_total;
  }
  double speed = particle_speed(p);
  double distance_cutoff = (S.time_cutoff < INFTY) ? (S.time_cutoff - p.time) * speed : INFTY;
  double distance = std::min({p.boundary.distance, p.collision_distance, distance_cutoff});
  for (int j = 0; j < p.n_coord; ++j)
    p.coord[j].r = p.coord[j].r + distance * p.coord[j].u;
  double dt = distance / speed;
  p.time += dt;
  if (!S.tallies.empty())
    score_tracklength_tally(S, p, distance);
  // src/particle.cpp:272-275
  if (S.eigenvalue)
    p.keff_tally_tracklength += p.wgt * distance * p.macro_nu_fission;
  if (distance == distance_cutoff)
    p.wgt = 0.0;
  if (p.trace && p.trace_n < p.trace_cap)
    p.trace[p.trace_n].dist = distance;
}

// src/particle.cpp:631-655
void cross_vacuum_bc(Particle& p)
{
  p.keff_tally_leakage += p.wgt;
  p.wgt = 0.0;
}

// src/particle.cpp:657-710
void cross_reflective_bc(Sim& S, Particle& p, Pos new_u)
{
  if (p.n_coord != 1) {
    mark_as_lost(S, p);
    return;
  }
  p.u() = new_u;
  p.coord[0].cell = p.cell_last[0];
  p.surface = -p.surface;
  p.n_coord = 1;
  if (!neighbor_list_find_cell(S, p)) {
    mark_as_lost(S, p);
    return;
  }
}

// src/particle.cpp:549-629
void cross_surface(Sim& S, Particle& p, const Surface& surf)
{
  if (surf.bc == 1) {
    cross_vacuum_bc(p);
    return;
  }
  if (surf.bc == 2) {
    // src/boundary_condition.cpp:38-47 ReflectiveBC::handle_particle
    Pos u = reflect(p.u(), surf_normal(surf, p.r()));
    u = u / u.norm();
    cross_reflective_bc(S, p, u);
    return;
  }
  if (neighbor_list_find_cell(S, p))
    return;
  p.n_coord = 1;
  bool found = exhaustive_find_cell(S, p);
  if (!found) {
    p.surface = SURFACE_NONE;
    p.n_coord = 1;
    p.r() = p.r() + TINY_BIT * p.u();
    if (!exhaustive_find_cell(S, p)) {
      mark_as_lost(S, p);
      return;
    }
  }
}

// src/particle.cpp:288-329
void event_cross_surface(Sim& S, Particle& p)
{
  for (int j = 0; j < p.n_coord; ++j)
    p.cell_last[j] = p.coord[j].cell;
  p.n_coord_last = p.n_coord;
  p.surface = p.boundary.surface;
  p.n_coord = p.boundary.coord_level;
  if (p.boundary.lattice_translation[0] != 0 || p.boundary.lattice_translation[1] != 0 ||
      p.boundary.lattice_translation[2] != 0) {
    cross_lattice(S, p, p.boundary);
  } else {
    const Surface& surf = S.surfaces[std::abs(p.surface) - 1];
    cross_surface(S, p, surf);
  }
}

// src/particle.cpp:331-415
void event_collide(Sim& S, Particle& p)
{
  // src/particle.cpp:333-337 collision estimate of k-effective
  if (S.eigenvalue)
    p.keff_tally_collision += p.wgt * p.macro_nu_fission / p.macro_total;
  p.surface = SURFACE_NONE;
  collision(S, p);
  // src/particle.cpp:361-364
  if (S.n_collision_tallies > 0) score_collision_tally(S, p);
  p.material_last = C_NONE;
  for (int j = 0; j < p.n_coord - 1; ++j)
    p.coord[j + 1].u = p.coord[j].u;
}

// src/particle.cpp:114-158
void from_source(Sim& S, Particle& p, const SourceSite& src)
{
  p.clear();
  p.surface = SURFACE_NONE;
  p.cell_born = C_NONE;
  p.material = C_NONE;
  p.n_collision = 0;
  p.wgt = src.wgt;
  p.wgt_last = src.wgt;
  p.r() = src.r;
  p.u() = src.u;
  p.r_last = src.r;
  p.u_last = src.u;
  p.E = src.E;
  p.E_last = p.E;
  p.time = src.time;
  p.time_last = src.time;
  p.surface = src.surf_id;  // surf_id holds the signed index+1 here
  (void)S;
}

// src/particle.cpp:417-473
bool event_revive_from_secondary(Sim& S, Particle& p)
{
  ++p.n_event;
  if (p.n_event == S.max_particle_events)
    p.wgt = 0.0;
  if (!p.alive()) {
    if (p.secondary_bank.empty())
      return false;
    from_source(S, p, p.secondary_bank.back());
    p.secondary_bank.pop_back();
    p.n_event = 0;
    return true;
  }
  return false;
}

// src/particle.cpp:475-512 (fixed source: leakage global tally)
void event_death(Sim& S, Particle& p)
{
#pragma omp atomic
  S.leakage += p.keff_tally_leakage;
  p.keff_tally_leakage = 0.0;
  if (S.eigenvalue) {
#pragma omp atomic
    S.k_abs += p.keff_tally_absorption;
#pragma omp atomic
    S.k_col += p.keff_tally_collision;
#pragma omp atomic
    S.k_tra += p.keff_tally_tracklength;
    p.keff_tally_absorption = p.keff_tally_collision = p.keff_tally_tracklength = 0.0;
    // src/particle.cpp:505-510: progeny count for the fission bank sort
    S.progeny_per_particle[p.id - 1] = p.n_progeny;
  }
}

// ------------------------------------------------------------------ source
// src/source.cpp:226-260 satisfies_spatial_constraints
bool satisfies_spatial_constraints(Sim& S, const Pos& r)
{
  Particle g;
  g.r() = r;
  g.u() = {0.0, 0.0, 1.0};
  if (!exhaustive_find_cell(S, g))
    return false;
  if (S.dom_type < 0 || S.dom_ids.empty())
    return true;
  if (S.dom_type == 1) {
    if (g.material == MATERIAL_VOID) return false;
    int64_t id = S.mat_id[g.material];
    return std::find(S.dom_ids.begin(), S.dom_ids.end(), id) != S.dom_ids.end();
  }
  for (int i = 0; i < g.n_coord; i++) {
    int64_t id = (S.dom_type == 0) ? S.cell_id[g.coord[i].cell] : -1;
    if (S.dom_type == 2) id = g.coord[i].universe;  // universe index
    if (std::find(S.dom_ids.begin(), S.dom_ids.end(), id) != S.dom_ids.end())
      return true;
  }
  return false;
}

// src/distribution.cpp:87-136 Discrete (alias) sampling
double sample_discrete(const Sim& S, uint64_t* seed)
{
  size_t n = S.en_par.size() / 2;
  if (n <= 1)
    return S.en_par[0];
  // Alias table construction, src/distribution.cpp:30-80 (Vose)
  std::vector<double> prob(n);
  std::vector<size_t> alias(n, 0);
  double sum = 0.0;
  for (size_t k = 0; k < n; ++k) sum += S.en_par[n + k];
  for (size_t k = 0; k < n; ++k) prob[k] = S.en_par[n + k] / sum * n;
  std::vector<size_t> large, small;
  for (size_t k = 0; k < n; ++k) (prob[k] > 1.0 ? large : small).push_back(k);
  while (!large.empty() && !small.empty()) {
    size_t j = small.back();
    size_t k = large.back();
    alias[j] = k;
    small.pop_back();
    prob[k] += prob[j] - 1.0;
    if (prob[k] < 1.0) {
      small.push_back(k);
      large.pop_back();
    }
  }
  size_t u = prn(seed) * n;
  if (prn(seed) < prob[u]) return S.en_par[u];
  return S.en_par[alias[u]];
}

// src/source.cpp:355-415 IndependentSource::sample
SourceSite sample_external_source(Sim& S, uint64_t* seed)
{
  SourceSite site;
  bool accepted = false;
  while (!accepted) {
    if (S.sp_type == 0) {
      site.r = {S.sp_par[0], S.sp_par[1], S.sp_par[2]};
    } else {
      double x = prn(seed);
      double y = prn(seed);
      double z = prn(seed);
      Pos xi {x, y, z};
      Pos ll {S.sp_par[0], S.sp_par[1], S.sp_par[2]};
      Pos ur {S.sp_par[3], S.sp_par[4], S.sp_par[5]};
      site.r = ll + xi * (ur - ll);
    }
    accepted = satisfies_spatial_constraints(S, site.r);
  }
  if (S.an_type == 0) {
    site.u = isotropic_direction(seed);
  } else {
    site.u = S.u_ref;
  }
  while (true) {
    site.E = (S.en_type == 0) ? sample_discrete(S, seed) : maxwell_spectrum(S.en_par[0], seed);
    if (site.E < S.energy_max)
      break;
  }
  site.time = 0.0;
  site.wgt = 1.0;
  return site;
}

// src/simulation.cpp:573-649 initialize_history (fixed source, first run)
void initialize_history(Sim& S, Particle& p, int batch, int64_t index_source)
{
  int64_t id = static_cast<int64_t>(batch - 1) * S.n_particles + index_source;
  if (S.eigenvalue) {
    // src/simulation.cpp:576-578: from the generation's source bank
    SourceSite site = S.source_bank[index_source - 1];
    site.surf_id = SURFACE_NONE;
    from_source(S, p, site);
  } else {
    uint64_t seed = init_seed(S.rng, id, STREAM_SOURCE);
    SourceSite site = sample_external_source(S, &seed);
    site.surf_id = SURFACE_NONE;
    from_source(S, p, site);
  }
  p.id = index_source;
  p.n_progeny = 0;
  p.lost = false;
  p.n_event = 0;
  p.n_split = 0;
  p.ww_factor = 0.0;
  p.wgt_born = p.wgt;
  init_particle_seeds(S.rng, id, p.seeds);
  p.stream = STREAM_TRACKING;
  p.wgt_ww_born = -1.0;
  apply_weight_windows(S, p);
#pragma omp atomic
  S.total_weight += p.wgt;
  for (auto& m : p.micro)
    m.last_E = 0.0;
}

// src/simulation.cpp:804-821 transport_history_based_single_particle
void transport_single(Sim& S, Particle& p)
{
  while (p.alive()) {
    event_calculate_xs(S, p);
    if (p.alive())
      event_advance(S, p);
    int kind = 0, sn = 0;
    double dist = p.trace && p.trace_n < p.trace_cap ? p.trace[p.trace_n].dist : 0.0;
    if (p.alive()) {
      if (p.collision_distance > p.boundary.distance) {
        kind = 1;
        sn = p.boundary.surface;
        event_cross_surface(S, p);
      } else if (p.alive()) {
        kind = 2;
        event_collide(S, p);
        sn = p.event_nuclide;
      }
    }
    trace_push(p, kind, sn, dist);
    event_revive_from_secondary(S, p);
  }
  event_death(S, p);
}

// ----------------------------------------------------------- sim building
void build(Sim& S, const Blob& B)
{
  const auto& si = B.I("settings_i");
  S.n_particles = si[0];
  S.n_batches = static_cast<int>(si[1]);
  S.n_inactive = static_cast<int>(si[2]);
  S.rng.master_seed = si[3];
  S.n_log_bins = static_cast<int>(si[4]);
  S.max_history_splits = si[5];
  S.ww_on = si[7] != 0;
  S.energy_cutoff = B.D("settings_d")[0];
  if (B.D("settings_d").size() > 1) S.time_cutoff = B.D("settings_d")[1];

  // nuclides
  const auto& off = B.I("nuc_off");
  const auto& en = B.D("nuc_energy");
  const auto& el = B.D("nuc_elastic");
  const auto& cap = B.D("nuc_capture");
  int n_nuc = static_cast<int>(off.size()) - 1;
  const auto& fis = B.D("nuc_fission");
  const auto& fis_i = B.I("nuc_fis_i");  // [fissionable, spectrum] per nuclide
  const auto& fis_d = B.D("nuc_fis_d");  // [nu0, nu1, sp0, sp1, u] per nuclide
  S.nuclides.resize(n_nuc);
  for (int i = 0; i < n_nuc; ++i) {
    Nuclide& nuc = S.nuclides[i];
    nuc.awr = B.D("nuc_awr")[i];
    nuc.kT = B.D("nuc_kT")[i];
    int G = static_cast<int>(off[i + 1] - off[i]);
    nuc.energy.assign(en.begin() + off[i], en.begin() + off[i + 1]);
    nuc.fissionable = fis_i[2 * i] != 0;
    nuc.spectrum = static_cast<int>(fis_i[2 * i + 1]);
    nuc.nu_c[0] = fis_d[5 * i];
    nuc.nu_c[1] = fis_d[5 * i + 1];
    nuc.sp[0] = fis_d[5 * i + 2];
    nuc.sp[1] = fis_d[5 * i + 3];
    nuc.u = fis_d[5 * i + 4];
    create_derived(nuc, el.data() + off[i], nuc.fissionable ? fis.data() + off[i] : nullptr, cap.data() + off[i], G);
  }
  const auto& eig = B.I("eig_i");  // [eigenvalue run, generations per batch]
  S.eigenvalue = eig[0] != 0;
  if (S.eigenvalue && eig[1] != 1) throw std::runtime_error("one generation per batch is supported");
  S.keff = B.D("eig_d")[0];
  // src/simulation.cpp:682-761 initialize_data
  S.energy_min = 0.0;
  S.energy_max = INFTY;
  for (auto& nuc : S.nuclides) {
    S.energy_min = std::max(S.energy_min, nuc.energy.front());
    S.energy_max = std::min(S.energy_max, nuc.energy.back());
  }
  for (auto& nuc : S.nuclides)
    init_grid(nuc, S.energy_min, S.energy_max, S.n_log_bins);
  S.energy_max_neutron = S.energy_max;  // data::energy_max[neutron]: the smallest grid maximum
  S.log_spacing = std::log(S.energy_max / S.energy_min) / S.n_log_bins;

  // materials: src/material.cpp:417-467 normalize_density (atom percents)
  const auto& moff = B.I("mat_off");
  int n_mat = static_cast<int>(moff.size()) - 1;
  S.materials.resize(n_mat);
  for (int m = 0; m < n_mat; ++m) {
    Material& mat = S.materials[m];
    double sum = 0.0;
    for (int64_t k = moff[m]; k < moff[m + 1]; ++k) {
      mat.nuclide.push_back(static_cast<int>(B.I("mat_nuc")[k]));
      mat.atom_density.push_back(B.D("mat_ao")[k]);
    }
    for (double v : mat.atom_density) sum += v;
    for (double& v : mat.atom_density) v /= sum;
    double density = B.D("mat_density")[m];
    for (double& v : mat.atom_density) v *= density;
  }
  S.mat_id.assign(B.I("mat_id").begin(), B.I("mat_id").end());

  // surfaces
  const auto& st = B.I("surf_type");
  S.surfaces.resize(st.size());
  for (size_t k = 0; k < st.size(); ++k) {
    Surface& s = S.surfaces[k];
    s.type = static_cast<int>(st[k]);
    for (int j = 0; j < 4; ++j) s.c[j] = B.D("surf_coeffs")[4 * k + j];
    s.bc = static_cast<int>(B.I("surf_bc")[k]);
    s.id = static_cast<int>(B.I("surf_id")[k]);
  }
  // cells
  const auto& cu = B.I("cell_univ");
  S.cells.resize(cu.size());
  for (size_t k = 0; k < cu.size(); ++k) {
    Cell& c = S.cells[k];
    c.id = static_cast<int>(B.I("cell_id")[k]);
    c.universe = static_cast<int>(cu[k]);
    c.fill_type = static_cast<int>(B.I("cell_ftype")[k]);
    c.fill = static_cast<int>(B.I("cell_fill")[k]);
    for (int64_t t = B.I("cell_tok_off")[k]; t < B.I("cell_tok_off")[k + 1]; ++t)
      c.expr.push_back(static_cast<int32_t>(B.I("cell_tok")[t]));
    c.simple = B.I("cell_simple")[k] != 0;
    c.translation = {B.D("cell_trans")[3 * k], B.D("cell_trans")[3 * k + 1], B.D("cell_trans")[3 * k + 2]};
  }
  S.cell_id.assign(B.I("cell_id").begin(), B.I("cell_id").end());
  const auto& uo = B.I("univ_cell_off");
  S.universes.resize(uo.size() - 1);
  for (size_t u = 0; u + 1 < uo.size(); ++u)
    for (int64_t k = uo[u]; k < uo[u + 1]; ++k)
      S.universes[u].push_back(static_cast<int>(B.I("univ_cells")[k]));
  S.root_universe = static_cast<int>(B.I("root_univ")[0]);
  const auto& lo = B.I("lat_univ_off");
  S.lattices.resize(lo.size() - 1);
  for (size_t l = 0; l + 1 < lo.size(); ++l) {
    Lattice& lat = S.lattices[l];
    for (int j = 0; j < 3; ++j) lat.n[j] = static_cast<int>(B.I("lat_n")[3 * l + j]);
    lat.ll = {B.D("lat_ll")[3 * l], B.D("lat_ll")[3 * l + 1], B.D("lat_ll")[3 * l + 2]};
    lat.pitch = {B.D("lat_pitch")[3 * l], B.D("lat_pitch")[3 * l + 1], B.D("lat_pitch")[3 * l + 2]};
    lat.is_3d = B.I("lat_is3d")[l] != 0;
    lat.outer = static_cast<int>(B.I("lat_outer")[l]);
    for (int64_t k = lo[l]; k < lo[l + 1]; ++k)
      lat.universes.push_back(static_cast<int>(B.I("lat_univ")[k]));
  }
  // coordinate depth: longest universe chain from the root
  std::function<int(int)> depth = [&](int u) -> int {
    int best = 1;
    for (int c : S.universes[u]) {
      const Cell& cell = S.cells[c];
      if (cell.fill_type == 1) best = std::max(best, 1 + depth(cell.fill));
      if (cell.fill_type == 2) {
        const Lattice& lat = S.lattices[cell.fill];
        for (int lu : lat.universes) best = std::max(best, 1 + depth(lu));
        if (lat.outer >= 0) best = std::max(best, 1 + depth(lat.outer));
      }
    }
    return best;
  };
  S.n_coord_levels = depth(S.root_universe);
  if (S.n_coord_levels > MAX_COORD) throw std::runtime_error("geometry too deep");
  S.cell_sqrtkT = std::sqrt(8.617333262e-5 * 293.6);

  // meshes
  const auto& nd = B.I("mesh_ndim");
  S.meshes.resize(nd.size());
  for (size_t k = 0; k < nd.size(); ++k) {
    Mesh& m = S.meshes[k];
    m.ndim = static_cast<int>(nd[k]);
    for (int j = 0; j < 3; ++j) {
      m.shape[j] = static_cast<int>(B.I("mesh_dim")[3 * k + j]);
      m.ll[j] = B.D("mesh_ll")[3 * k + j];
      m.ur[j] = B.D("mesh_ur")[3 * k + j];
      m.width[j] = B.D("mesh_width")[3 * k + j];
    }
  }
  // filters and tallies; src/tallies/tally.cpp:503-516 set_strides
  const auto& ft = B.I("filt_type");
  S.filters.resize(ft.size());
  for (size_t k = 0; k < ft.size(); ++k) {
    Filter& f = S.filters[k];
    f.type = static_cast<int>(ft[k]);
    f.mesh = static_cast<int>(B.I("filt_mesh")[k]);
    f.nbins = static_cast<int>(B.I("filt_nbins")[k]);
    for (int64_t j = B.I("filt_eoff")[k]; j < B.I("filt_eoff")[k + 1]; ++j)
      f.bins.push_back(B.D("filt_e")[j]);
    for (int64_t j = B.I("filt_ioff")[k]; j < B.I("filt_ioff")[k + 1]; ++j)
      f.ids.push_back(static_cast<int>(B.I("filt_ids")[j]));
  }
  const auto& tid = B.I("tal_id");
  S.tallies.resize(tid.size());
  for (size_t k = 0; k < tid.size(); ++k) {
    Tally& t = S.tallies[k];
    t.id = static_cast<int>(tid[k]);
    for (int64_t j = B.I("tal_filt_off")[k]; j < B.I("tal_filt_off")[k + 1]; ++j)
      t.filters.push_back(static_cast<int>(B.I("tal_filt")[j]));
    for (int64_t j = B.I("tal_score_off")[k]; j < B.I("tal_score_off")[k + 1]; ++j)
      t.scores.push_back(static_cast<int>(B.I("tal_score")[j]));
    t.estimator = static_cast<int>(B.I("tal_est")[k]);
    if (t.estimator == 1) ++S.n_collision_tallies;
    t.strides.assign(t.filters.size(), 1);
    int64_t stride = 1;
    for (int i = static_cast<int>(t.filters.size()) - 1; i >= 0; --i) {
      t.strides[i] = static_cast<int>(stride);
      stride *= S.filters[t.filters[i]].nbins;
    }
    t.n_filter_bins = stride;
    t.results.assign(static_cast<size_t>(stride) * t.scores.size() * 3, 0.0);
  }

  // source
  const auto& sr = B.I("src_i");
  S.sp_type = static_cast<int>(sr[0]);
  S.an_type = static_cast<int>(sr[1]);
  S.en_type = static_cast<int>(sr[2]);
  S.dom_type = static_cast<int>(sr[3]);
  S.sp_par = B.D("src_space");
  const auto& ur = B.D("src_uref");
  S.u_ref = {ur[0], ur[1], ur[2]};
  S.en_par = B.D("src_energy");
  S.strength = B.D("src_strength")[0];
  S.dom_ids = B.I("src_dom_ids");

  // weight windows
  const auto& wi = B.I("ww_i");
  if (wi[0] >= 0) {
    S.ww.mesh = static_cast<int>(wi[0]);
    S.ww.max_split = static_cast<int>(wi[2]);
    S.ww.survival_ratio = B.D("ww_d")[0];
    S.ww.max_lb_ratio = B.D("ww_d")[1];
    S.ww.weight_cutoff = B.D("ww_d")[2];
    S.ww.energy_bounds = B.D("ww_e");
    S.ww.lower = B.D("ww_lower");
    S.ww.upper = B.D("ww_upper");
  } else {
    S.ww_on = false;
  }
}

// src/tallies/tally.cpp:821-880 Tally::accumulate
// ------------------------------------------------------------ eigenvalue
// src/source.cpp:601-615 initialize_source (first generation) and
// src/simulation.cpp:507-520 initialize_generation
void eigen_begin_batch(Sim& S, int batch)
{
  if (batch == 1) {
    S.source_bank.assign(S.n_particles, SourceSite {});
    for (int64_t i = 0; i < S.n_particles; ++i) {
      uint64_t seed = init_seed(S.rng, i + 1, STREAM_SOURCE);
      S.source_bank[i] = sample_external_source(S, &seed);
    }
    S.fission_bank_cap = 3 * S.n_particles;
    S.fission_bank.assign(S.fission_bank_cap, SourceSite {});
  }
  S.n_fission_sites = 0;
  S.fission_bank_full = 0;
  S.progeny_per_particle.assign(S.n_particles, 0);
  S.keff_generation = S.gt[2][0];
}

// src/bank.cpp:76-135 sort_fission_bank: exclusive scan of the progeny
// counts, each site to its parent's offset plus its progeny number
void sort_fission_bank(Sim& S)
{
  std::vector<int64_t> off(S.progeny_per_particle.size());
  int64_t acc = 0;
  for (size_t i = 0; i < off.size(); ++i) {
    off[i] = acc;
    acc += S.progeny_per_particle[i];
  }
  std::vector<SourceSite> sorted(S.n_fission_sites);
  for (int64_t i = 0; i < S.n_fission_sites; ++i) {
    const SourceSite& site = S.fission_bank[i];
    int64_t idx = off[site.parent_id - 1] + site.progeny_id;
    if (idx >= S.n_fission_sites)
      throw std::runtime_error("Mismatch detected between sum of all particle progeny and shared fission bank size.");
    sorted[idx] = site;
  }
  std::copy(sorted.begin(), sorted.end(), S.fission_bank.begin());
}

// src/eigenvalue.cpp:86-365 synchronize_bank on one rank: uniform combing
// of n_particles teeth over the sorted bank, the comb's offset drawn from
// the tracking stream of the generation's id
void synchronize_bank(Sim& S, int batch)
{
  int64_t start = 0;
  int64_t finish = S.n_fission_sites;
  int64_t total = finish;
  if (S.n_fission_sites == 0) throw std::runtime_error("No fission sites banked on MPI rank 0");
  std::vector<SourceSite> temp_sites(3 * S.n_particles);
  int64_t index_temp = 0;
  int64_t id = 0 + batch;  // total_gen + overall_generation() with one generation per batch
  uint64_t seed = init_seed(S.rng, id, STREAM_TRACKING);
  double teeth_distance = static_cast<double>(total) / S.n_particles;
  double teeth_offset = prn(&seed) * teeth_distance;
  int64_t end = start + S.n_fission_sites;
  int64_t tooth_start = std::ceil((start - teeth_offset) / teeth_distance);
  int64_t tooth_end = std::floor((end - teeth_offset) / teeth_distance) + 1;
  double tooth = tooth_start * teeth_distance + teeth_offset;
  for (int64_t i = tooth_start; i < tooth_end; i++) {
    int64_t idx = std::floor(tooth) - start;
    temp_sites[index_temp] = S.fission_bank[idx];
    ++index_temp;
    tooth += teeth_distance;
  }
  if (index_temp < S.n_particles) throw std::runtime_error("the comb selected fewer sites than particles");
  std::copy(temp_sites.begin(), temp_sites.begin() + S.n_particles, S.source_bank.begin());
}

// src/eigenvalue.cpp:367-418 calculate_average_keff (one generation per
// batch, no confidence-interval t-value)
void calculate_average_keff(Sim& S, int batch)
{
  int i = batch - 1;
  int n = batch > S.n_inactive ? S.n_realizations + 1 : 0;
  if (n <= 0) {
    S.keff = S.k_generation[i];
  } else {
    S.k_sum[0] += S.k_generation[i];
    S.k_sum[1] += std::pow(S.k_generation[i], 2);
    S.keff = S.k_sum[0] / n;
    if (n > 1) {
      double t_value = 1.0;
      S.keff_std = t_value * std::sqrt((S.k_sum[1] / n - std::pow(S.keff, 2)) / (n - 1));
      if (!std::isfinite(S.keff_std)) S.keff_std = 0.0;
    }
  }
}

// src/simulation.cpp:522-570 finalize_generation and
// src/eigenvalue.cpp:50-84 calculate_generation_keff
void eigen_end_batch(Sim& S, int batch)
{
  if (S.fission_bank_full) throw std::runtime_error("The shared fission bank is full.");
  S.gt[0][0] += S.k_col;
  S.gt[1][0] += S.k_abs;
  S.gt[2][0] += S.k_tra;
  S.k_col = S.k_abs = S.k_tra = 0.0;
  sort_fission_bank(S);
  synchronize_bank(S, batch);
  double kg = S.gt[2][0] - S.keff_generation;
  kg /= S.n_particles;
  S.k_generation.push_back(kg);
  calculate_average_keff(S, batch);
}

void accumulate(Sim& S)
{
  double norm = S.strength / (static_cast<double>(S.n_particles) * 1);
  for (auto& t : S.tallies) {
    t.n_realizations += 1;
    size_t n = t.results.size() / 3;
    for (size_t i = 0; i < n; ++i) {
      double val = t.results[3 * i] * norm;
      t.results[3 * i] = 0.0;
      t.results[3 * i + 1] += val;
      t.results[3 * i + 2] += val * val;
    }
  }
  double l = S.leakage / S.total_weight;
  S.leak_s1 += l;
  S.leak_s2 += l * l;
  S.leakage = 0.0;
  S.total_weight = 0.0;
}

// src/tallies/tally.cpp:1059-1100 accumulate_tallies and
// src/simulation.cpp:402-418 finalize_batch for an eigenvalue run: user
// tallies score only in active batches; global tallies (normalised by the
// source weight) accumulate every batch and are reset, with the realization
// count, after each inactive one
void accumulate_eigen(Sim& S, int batch)
{
  S.n_realizations += 1;
  bool active = batch > S.n_inactive;
  if (active) {
    double k_col = S.gt[0][0] / S.total_weight;
    double k_abs = S.gt[1][0] / S.total_weight;
    double k_tra = S.gt[2][0] / S.total_weight;
    S.k_col_abs += k_col * k_abs;
    S.k_col_tra += k_col * k_tra;
    S.k_abs_tra += k_abs * k_tra;
  }
  for (int i = 0; i < 3; ++i) {
    double val = S.gt[i][0] / S.total_weight;
    S.gt[i][0] = 0.0;
    S.gt[i][1] += val;
    S.gt[i][2] += val * val;
  }
  if (active) {
    accumulate(S);
  } else {
    for (auto& t : S.tallies)
      for (size_t i = 0; i < t.results.size(); i += 3) t.results[i] = 0.0;
    S.leakage = 0.0;
    S.total_weight = 0.0;
    for (auto& row : S.gt) row[0] = row[1] = row[2] = 0.0;
    S.n_realizations = 0;
  }
}

struct Handle {
  Sim S;
  std::vector<TraceRec> trace;
  std::vector<int32_t> trace_n;
  int64_t trace_hist = 0;
  int trace_cap = 0;
  int trace_batch = 1;
  std::string err;
};

}  // namespace orc

using namespace orc;

extern "C" {

void* oracle_create(const uint8_t* blob, size_t n, char* err, int errlen)
{
  try {
    auto* h = new Handle();
    build(h->S, parse_blob(blob, n));
    return h;
  } catch (const std::exception& e) {
    if (err && errlen > 0) std::snprintf(err, errlen, "%s", e.what());
    return nullptr;
  }
}

void oracle_destroy(void* h) { delete static_cast<Handle*>(h); }

// Record per-event traces for the first n_hist particle ids of the next batch.
void oracle_set_trace(void* hv, int64_t n_hist, int cap, int batch)
{
  auto* h = static_cast<Handle*>(hv);
  h->trace_batch = batch;
  h->trace_hist = n_hist;
  h->trace_cap = cap;
  h->trace.assign(static_cast<size_t>(n_hist) * cap, TraceRec {});
  h->trace_n.assign(n_hist, 0);
}

const void* oracle_trace_data(void* hv) { return static_cast<Handle*>(hv)->trace.data(); }
const int32_t* oracle_trace_counts(void* hv) { return static_cast<Handle*>(hv)->trace_n.data(); }

// Transport particles [first, first+count) (1-based source index) of `batch`.
// mode 0: history-based loop (src/simulation.cpp:823-831);
// mode 1: event-based loop with the reference's five queues
// (src/simulation.cpp:833-883, src/event.cpp:62-177).
int oracle_transport(void* hv, int batch, int64_t first, int64_t count, int mode, int threads, int64_t in_flight)
{
  auto* h = static_cast<Handle*>(hv);
  Sim& S = h->S;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  size_t n_nuc = S.nuclides.size();
  try {
    if (mode == 0) {
#pragma omp parallel
      {
        Particle p;
        p.micro.assign(n_nuc, MicroXS {});
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = first; i < first + count; ++i) {
          p.secondary_bank.clear();
          p.trace = nullptr;
          initialize_history(S, p, batch, i);
          if (batch == h->trace_batch && i <= h->trace_hist) {
            p.trace = &h->trace[static_cast<size_t>(i - 1) * h->trace_cap];
            p.trace_cap = h->trace_cap;
            p.trace_n = 0;
          }
          transport_single(S, p);
          if (p.trace) h->trace_n[i - 1] = p.trace_n;
        }
      }
    } else {
      // event-based: queues hold particle buffer indices
      int64_t remaining = count, offset = first;
      int64_t cap = in_flight > 0 ? in_flight : 100000;
      std::vector<Particle> parts(std::min(cap, count));
      for (auto& p : parts) p.micro.assign(n_nuc, MicroXS {});
      std::vector<int64_t> q_xs, q_adv, q_surf, q_coll;
      while (remaining > 0) {
        int64_t n = std::min(remaining, cap);
        q_xs.clear();
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
          parts[i].secondary_bank.clear();
          parts[i].trace = nullptr;
          initialize_history(S, parts[i], batch, offset + i);
        }
        for (int64_t i = 0; i < n; ++i) q_xs.push_back(i);
        while (!q_xs.empty()) {
          int64_t nx = static_cast<int64_t>(q_xs.size());
#pragma omp parallel for schedule(static)
          for (int64_t k = 0; k < nx; ++k) event_calculate_xs(S, parts[q_xs[k]]);
          q_adv.swap(q_xs);
          q_xs.clear();
          int64_t na = static_cast<int64_t>(q_adv.size());
          std::vector<char> to_surf(na, 0), alive(na, 0);
#pragma omp parallel for schedule(static)
          for (int64_t k = 0; k < na; ++k) {
            Particle& p = parts[q_adv[k]];
            event_advance(S, p);
            alive[k] = p.alive();
            to_surf[k] = p.collision_distance > p.boundary.distance;
          }
          q_surf.clear();
          q_coll.clear();
          for (int64_t k = 0; k < na; ++k) {
            if (!alive[k]) continue;
            (to_surf[k] ? q_surf : q_coll).push_back(q_adv[k]);
          }
          std::vector<char> keep_s(q_surf.size(), 0), keep_c(q_coll.size(), 0);
#pragma omp parallel for schedule(static)
          for (int64_t k = 0; k < static_cast<int64_t>(q_surf.size()); ++k) {
            Particle& p = parts[q_surf[k]];
            event_cross_surface(S, p);
            event_revive_from_secondary(S, p);
            keep_s[k] = p.alive();
          }
#pragma omp parallel for schedule(static)
          for (int64_t k = 0; k < static_cast<int64_t>(q_coll.size()); ++k) {
            Particle& p = parts[q_coll[k]];
            event_collide(S, p);
            event_revive_from_secondary(S, p);
            keep_c[k] = p.alive();
          }
          for (size_t k = 0; k < q_surf.size(); ++k) if (keep_s[k]) q_xs.push_back(q_surf[k]);
          for (size_t k = 0; k < q_coll.size(); ++k) if (keep_c[k]) q_xs.push_back(q_coll[k]);
        }
        for (int64_t i = 0; i < n; ++i) event_death(S, parts[i]);
        remaining -= n;
        offset += n;
      }
    }
  } catch (const std::exception& e) {
    h->err = e.what();
    return -1;
  }
  return 0;
}

int oracle_accumulate(void* hv)
{
  accumulate(static_cast<Handle*>(hv)->S);
  return 0;
}

// Eigenvalue run: before the batch's transport (first batch: initial source
// bank from the external source), after it (fission bank sort, comb,
// generation and average k), and the batch's accumulation.
int oracle_eigen_begin(void* hv, int batch)
{
  auto* h = static_cast<Handle*>(hv);
  try {
    eigen_begin_batch(h->S, batch);
  } catch (const std::exception& e) {
    h->err = e.what();
    return -1;
  }
  return 0;
}

int oracle_eigen_end(void* hv, int batch)
{
  auto* h = static_cast<Handle*>(hv);
  try {
    eigen_end_batch(h->S, batch);
    accumulate_eigen(h->S, batch);
  } catch (const std::exception& e) {
    h->err = e.what();
    return -1;
  }
  return 0;
}

// [keff, keff_std, n_realizations, fission sites of the last generation,
//  K_COLLISION / K_ABSORPTION / K_TRACKLENGTH (SUM, SUM_SQ), k_col_abs,
//  k_col_tra, k_abs_tra] and the generation k values (k_gen, up to n_gen)
int oracle_keff(void* hv, double* out, double* k_gen, int n_gen)
{
  Sim& S = static_cast<Handle*>(hv)->S;
  out[0] = S.keff;
  out[1] = S.keff_std;
  out[2] = S.n_realizations;
  out[3] = static_cast<double>(S.n_fission_sites);
  for (int i = 0; i < 3; ++i) {
    out[4 + 2 * i] = S.gt[i][1];
    out[5 + 2 * i] = S.gt[i][2];
  }
  out[10] = S.k_col_abs;
  out[11] = S.k_col_tra;
  out[12] = S.k_abs_tra;
  int n = static_cast<int>(S.k_generation.size());
  for (int i = 0; i < n && i < n_gen; ++i) k_gen[i] = S.k_generation[i];
  return n;
}

// src/eigenvalue.cpp:420-579 openmc_get_keff: k_combined[0..1]
void oracle_keff_combined(void* hv, double* k_combined)
{
  Sim& S = static_cast<Handle*>(hv)->S;
  k_combined[0] = 0.0;
  k_combined[1] = 0.0;
  if (S.n_realizations <= 3) {
    k_combined[0] = S.keff;
    k_combined[1] = S.keff_std;
    if (S.n_realizations <= 1) k_combined[1] = std::numeric_limits<double>::infinity();
    return;
  }
  int64_t n = S.n_realizations;
  std::array<double, 3> kv {};
  double cov[3][3] = {};
  kv[0] = S.gt[0][1] / n;
  kv[1] = S.gt[1][1] / n;
  kv[2] = S.gt[2][1] / n;
  cov[0][0] = (S.gt[0][2] - n * kv[0] * kv[0]) / (n - 1);
  cov[1][1] = (S.gt[1][2] - n * kv[1] * kv[1]) / (n - 1);
  cov[2][2] = (S.gt[2][2] - n * kv[2] * kv[2]) / (n - 1);
  cov[0][1] = (S.k_col_abs - n * kv[0] * kv[1]) / (n - 1);
  cov[0][2] = (S.k_col_tra - n * kv[0] * kv[2]) / (n - 1);
  cov[1][2] = (S.k_abs_tra - n * kv[1] * kv[2]) / (n - 1);
  cov[1][0] = cov[0][1];
  cov[2][0] = cov[0][2];
  cov[2][1] = cov[1][2];
  int i, j;
  bool use_three = false;
  if ((std::abs(kv[0] - kv[1]) / kv[0] < FP_REL_PRECISION) &&
      (std::abs(cov[0][0] - cov[1][1]) / cov[0][0] < FP_REL_PRECISION)) {
    i = 0; j = 2;
  } else if ((std::abs(kv[0] - kv[2]) / kv[0] < FP_REL_PRECISION) &&
             (std::abs(cov[0][0] - cov[2][2]) / cov[0][0] < FP_REL_PRECISION)) {
    i = 0; j = 1;
  } else if ((std::abs(kv[1] - kv[2]) / kv[1] < FP_REL_PRECISION) &&
             (std::abs(cov[1][1] - cov[2][2]) / cov[1][1] < FP_REL_PRECISION)) {
    i = 0; j = 1;
  } else {
    use_three = true;
    i = j = 0;
  }
  if (use_three) {
    double g = 0.0;
    std::array<double, 3> Ssum {};
    for (int l = 0; l < 3; ++l) {
      int k;
      switch (l) {
      case 0: i = 0; j = 1; k = 2; break;
      case 1: i = 1; j = 2; k = 0; break;
      default: i = 2; j = 0; k = 1; break;
      }
      double f = cov[j][j] * (cov[k][k] - cov[i][k]) - cov[k][k] * cov[i][j] +
                 cov[j][k] * (cov[i][j] + cov[i][k] - cov[j][k]);
      Ssum[0] += f * cov[0][l];
      Ssum[1] += (cov[j][j] + cov[k][k] - 2.0 * cov[j][k]) * kv[l] * kv[l];
      Ssum[2] += (cov[k][k] + cov[i][j] - cov[j][k] - cov[i][k]) * kv[l] * kv[j];
      k_combined[0] += f * kv[l];
      g += f;
    }
    for (auto& v : Ssum) v *= (n - 1);
    Ssum[0] *= (n - 1) * (n - 1);
    k_combined[0] /= g;
    g *= (n - 1) * (n - 1);
    k_combined[1] = std::sqrt(Ssum[0] / (g * n * (n - 3)) * (1 + n * ((Ssum[1] - 2 * Ssum[2]) / g)));
  } else {
    double f = kv[i] - kv[j];
    double g = cov[i][i] + cov[j][j] - 2.0 * cov[i][j];
    k_combined[0] = kv[i] - (cov[i][i] - cov[i][j]) / g * f;
    k_combined[1] = (cov[i][i] * cov[j][j] - cov[i][j] * cov[i][j]) * (g + n * f * f) / (n * (n - 2) * g * g);
    k_combined[1] = std::sqrt(k_combined[1]);
  }
}

// The source bank of the coming generation: n x [x, y, z, u, v, w, E, wgt]
int64_t oracle_source_bank(void* hv, double* out, int64_t n)
{
  Sim& S = static_cast<Handle*>(hv)->S;
  int64_t m = std::min<int64_t>(n, static_cast<int64_t>(S.source_bank.size()));
  for (int64_t i = 0; i < m; ++i) {
    const SourceSite& s = S.source_bank[i];
    double* o = out + 8 * i;
    o[0] = s.r.x; o[1] = s.r.y; o[2] = s.r.z;
    o[3] = s.u.x; o[4] = s.u.y; o[5] = s.u.z;
    o[6] = s.E; o[7] = s.wgt;
  }
  return m;
}

int oracle_n_tallies(void* hv) { return static_cast<int>(static_cast<Handle*>(hv)->S.tallies.size()); }

int64_t oracle_tally_size(void* hv, int t)
{
  return static_cast<int64_t>(static_cast<Handle*>(hv)->S.tallies[t].results.size());
}

const double* oracle_tally_results(void* hv, int t) { return static_cast<Handle*>(hv)->S.tallies[t].results.data(); }

void oracle_globals(void* hv, double* out)
{
  Sim& S = static_cast<Handle*>(hv)->S;
  out[0] = S.leak_s1;
  out[1] = S.leak_s2;
  out[2] = static_cast<double>(S.n_lost);
  out[3] = S.total_weight;
  out[4] = S.energy_min;
  out[5] = S.energy_max;
  out[6] = S.log_spacing;
}

// Macroscopic XS (total, absorption) and grid-index hash for (material, E) pairs.
void oracle_macro_xs(void* hv, int64_t n, const int32_t* mat, const double* E,
  double* total, double* absorption, int32_t* grid_hash)
{
  Sim& S = static_cast<Handle*>(hv)->S;
  Particle p;
  p.micro.assign(S.nuclides.size(), MicroXS {});
  for (int64_t i = 0; i < n; ++i) {
    for (auto& m : p.micro) m.last_E = 0.0;
    p.E = E[i];
    p.material = mat[i];
    material_calculate_xs(S, p);
    total[i] = p.macro_total;
    absorption[i] = p.macro_absorption;
    grid_hash[i] = p.trace_grid;
  }
}

// Per-nuclide hash-window index tables (for checking the product's init_grid).
int oracle_grid_index(void* hv, int nuc, int32_t* out, int n)
{
  Sim& S = static_cast<Handle*>(hv)->S;
  const auto& g = S.nuclides[nuc].grid_index;
  int m = std::min<int>(n, static_cast<int>(g.size()));
  for (int i = 0; i < m; ++i) out[i] = g[i];
  return static_cast<int>(g.size());
}

const char* oracle_error(void* hv) { return static_cast<Handle*>(hv)->err.c_str(); }

// ---- functions pinned against tests/cpp_unit_tests/test_math.cpp
double oracle_prn(uint64_t* seed) { return prn(seed); }
uint64_t oracle_future_seed(uint64_t n, uint64_t seed) { return future_seed(n, seed); }
uint64_t oracle_init_seed(int64_t id, int offset, int64_t master, uint64_t stride)
{
  RngConfig rc;
  rc.master_seed = master;
  rc.stride = stride;
  return init_seed(rc, id, offset);
}
int64_t oracle_lower_bound_index(const double* first, int64_t n, double value)
{
  return lower_bound_index(first, first + n, value);
}
double oracle_maxwell_spectrum(double T, uint64_t* seed) { return maxwell_spectrum(T, seed); }
double oracle_watt_spectrum(double a, double b, uint64_t* seed) { return watt_spectrum(a, b, seed); }
void oracle_rotate_angle(double* uvw, double mu, const double* phi, uint64_t* seed)
{
  Pos u = rotate_angle({uvw[0], uvw[1], uvw[2]}, mu, phi, seed);
  uvw[0] = u.x;
  uvw[1] = u.y;
  uvw[2] = u.z;
}

// ---- macroscopic-XS lookup microbenchmark restatement: the 5-column row
// lookup of src/material.cpp:829-901 + src/nuclide.cpp:724-775 on flat tables
// energy [n_nuc][G], xs [n_nuc][G][5]; hash tables built by init_grid.
struct XSB {
  int n_nuc, G, M;
  double e_min, e_max, log_spacing;
  std::vector<double> energy, xs;
  std::vector<int> grid_index;  // [n_nuc][M+1]
  std::vector<int> mat_off, mat_nuc;
  std::vector<double> mat_dens;
};

void* oracle_xsb_create(int n_nuc, int G, const double* energy, const double* xs,
  int n_mat, const int32_t* mat_off, const int32_t* mat_nuc, const double* mat_dens, int M)
{
  auto* x = new XSB();
  x->n_nuc = n_nuc;
  x->G = G;
  x->M = M;
  x->energy.assign(energy, energy + static_cast<size_t>(n_nuc) * G);
  x->xs.assign(xs, xs + static_cast<size_t>(n_nuc) * G * 5);
  x->mat_off.assign(mat_off, mat_off + n_mat + 1);
  x->mat_nuc.assign(mat_nuc, mat_nuc + mat_off[n_mat]);
  x->mat_dens.assign(mat_dens, mat_dens + mat_off[n_mat]);
  x->e_min = 0.0;
  x->e_max = INFTY;
  for (int i = 0; i < n_nuc; ++i) {
    x->e_min = std::max(x->e_min, x->energy[static_cast<size_t>(i) * G]);
    x->e_max = std::min(x->e_max, x->energy[static_cast<size_t>(i) * G + G - 1]);
  }
  x->grid_index.resize(static_cast<size_t>(n_nuc) * (M + 1));
  for (int i = 0; i < n_nuc; ++i) {
    Nuclide nuc;
    nuc.energy.assign(x->energy.begin() + static_cast<size_t>(i) * G, x->energy.begin() + static_cast<size_t>(i + 1) * G);
    init_grid(nuc, x->e_min, x->e_max, M);
    std::copy(nuc.grid_index.begin(), nuc.grid_index.end(), x->grid_index.begin() + static_cast<size_t>(i) * (M + 1));
  }
  x->log_spacing = std::log(x->e_max / x->e_min) / M;
  return x;
}

void oracle_xsb_destroy(void* x) { delete static_cast<XSB*>(x); }

void oracle_xsb_grid_index(void* xv, int32_t* out)
{
  auto* x = static_cast<XSB*>(xv);
  for (size_t i = 0; i < x->grid_index.size(); ++i) out[i] = x->grid_index[i];
}

void oracle_xsb_lookup(void* xv, int64_t n, const int32_t* mat, const double* Ein,
  double* out /*[n][5]*/, int32_t* grid_hash, int threads)
{
  auto* x = static_cast<XSB*>(xv);
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < n; ++k) {
    double E = Ein[k];
    int m = mat[k];
    int i_log = std::log(E / x->e_min) / x->log_spacing;
    i_log = std::min(std::max(i_log, 0), x->M - 1);
    double macro[5] = {0, 0, 0, 0, 0};
    uint32_t h = 0;
    for (int j = x->mat_off[m]; j < x->mat_off[m + 1]; ++j) {
      int nuc = x->mat_nuc[j];
      const double* e = &x->energy[static_cast<size_t>(nuc) * x->G];
      const int* gi = &x->grid_index[static_cast<size_t>(nuc) * (x->M + 1)];
      int i_grid;
      if (E < e[0]) {
        i_grid = 0;
      } else if (E > e[x->G - 1]) {
        i_grid = x->G - 2;
      } else {
        int i_low = gi[i_log];
        int i_high = gi[i_log + 1] + 1;
        i_grid = i_low + static_cast<int>(lower_bound_index(&e[i_low], &e[i_high], E));
      }
      if (e[i_grid] == e[i_grid + 1])
        ++i_grid;
      double f = (E - e[i_grid]) / (e[i_grid + 1] - e[i_grid]);
      const double* row = &x->xs[(static_cast<size_t>(nuc) * x->G + i_grid) * 5];
      double dens = x->mat_dens[j];
      for (int c = 0; c < 5; ++c)
        macro[c] += dens * ((1.0 - f) * row[c] + f * row[c + 5]);
      h = h * 31u + static_cast<uint32_t>(i_grid);
    }
    for (int c = 0; c < 5; ++c) out[5 * k + c] = macro[c];
    if (grid_hash) grid_hash[k] = static_cast<int32_t>(h);
  }
}

}  // extern "C"
