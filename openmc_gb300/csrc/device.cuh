// Device-side model layout and the per-particle physics/geometry functions of
// the event-based transport path.  Every function restates the reference
// function cited beside it with the same floating-point operation order; the
// library is compiled with -fmad=false so that no multiply-add is fused, and
// the only differences to a CPU build come from the device log/sin/cos.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fp64_int.cuh"
#include "transport.h"

// Each build of the transport kernels for a maximum coordinate depth lives
// in its own namespace (omc::l2, omc::l4) so that both link into one library.
#ifndef OMC_NS
#define OMC_NS l4
#endif
namespace omc {
namespace OMC_NS {

#ifndef OMC_MAXL
#define OMC_MAXL 4
#endif
constexpr int MAXL = OMC_MAXL;  // coordinate levels held per particle
constexpr double INFTY = 1.7976931348623157e308;  // numeric_limits<double>::max()
constexpr double PI = 3.141592653589793238462643383279502884;
constexpr double TINY_BIT = 1e-8;
constexpr double FP_PRECISION = 1e-14;
constexpr double FP_REL_PRECISION = 1e-5;
constexpr double FP_COINCIDENT = 1e-12;
constexpr double MASS_NEUTRON_EV = 939.56542052e6;
constexpr double C_LIGHT = 2.99792458e10;  // cm/s
constexpr int C_NONE = -1;
constexpr int SURFACE_NONE = 0;
constexpr uint64_t PRN_MULT = 6364136223846793005ULL;
constexpr uint64_t PRN_ADD = 1442695040888963407ULL;


struct DSurface {
  double c[4];
  double rr;  // radius squared (cylinders, spheres), the product the distance and sense expressions form
  int type, bc;
};

struct DCell {
  double tr[3];
  int universe, fill_type, fill, tok_off, tok_len, simple;
};

// FP64 cross-section row of one grid point (32 B, two 16-byte loads): the
// create_derived columns the transport reads (fission and nu-fission are 0
// for a nuclide without MT 18)
struct alignas(16) XsRow64 {
  double total, absorption, fission, nu_fission;
};

// Fission neutron data of a nuclide (MT 18, prompt product): yield
// polynomial nu0 + nu1 E, spectrum 1 Maxwell (p0 = theta) or 2 Watt (a, b),
// restriction energy u
struct DFission {
  double nu0, nu1, p0, p1, u;
  int spectrum, pad;
};

// One site of the fission bank (SourceSite of src/particle_data.h:43-57 for
// a prompt fission neutron: weight 1, the parent's time, on no surface)
struct DFissionSite {
  double r[3], u[3], E, time;
  long long parent;  // source index of the parent history (1-based)
  int progeny, pad;
};

struct DLattice {
  double ll[3], pitch[3];
  double half[3];  // 0.5 x pitch (exact)
  int n[3];
  int is3d, outer, univ_off;
};

struct DMesh {
  double ll[3], width[3];
  float inv_width32[3];  // 1 / width rounded to FP32, for the FP32 index pre-test
  float width32[3];      // width rounded to FP32 (the FP32-table mode track walk)
  int shape[3];
  int ndim;
};

struct DFilter {
  int type, mesh, nbins, e_off;
  int i_off;  // cell / material filters: offset of the bins' indices in DModel::fids
};

struct DTally {
  long long value_off;
  int estimator;  // 0 track length, 1 collision
  int nfilt, nscore;
  int filt[3], stride[3];
  int score[4];
};

struct DModel {
  // geometry
  const DSurface* surf;
  const DCell* cell;
  const int* tok;
  const int* univ_off;
  const int* univ_cells;
  const DLattice* lat;
  const int* lat_univ;
  int n_surf, n_cell, n_univ, n_lat, root_univ, n_coord_levels;
  // nuclear data
  const long long* nuc_off;  // grid offsets
  const double* energy;
  const XsRow64* xs64;  // (total, absorption, elastic, 0) per grid point
  const float4* xs32;
  const int* grid_index;  // [n_nuc][M+1]
  const double* awr;
  const double* kT;
  const int* mat_off;
  const int* mat_nuc;
  const double* mat_dens;
  const float* mat_dens32;
  const DFission* fis;  // per nuclide (eigenvalue runs)
  int n_nuc, n_mat, M, xs_fp32;
  // eigenvalue run: the running k-effective the fission sites are sampled
  // with, and data::energy_max[neutron] (fission energies at or above it
  // are resampled)
  int eigen;
  double keff, e_max_neutron;
  double e_min, e_max, log_spacing;
  float log_emin32, inv_spacing32;  // FP32 log(e_min) and 1 / log_spacing for the hash-bin pre-test
  // source
  int sp_type, an_type, en_type, dom_type, n_en, n_dom;
  double sp[6], uref[3];
  double en_x[8], en_prob[8];
  int en_alias[8];
  const int* dom_ids;
  const int* mat_id;
  const int* cell_id;
  // tallies
  int n_tally;
  int n_tally_tracklength, n_tally_collision;
  // what a deferred track record must carry beyond position, direction,
  // length, weight and energy: the macroscopic XS (a track-length tally
  // scores total or absorption), the cells of every level (a cell filter),
  // the material (a material filter)
  int trk_xs, trk_cells, trk_mat;
  const DTally* tally;
  const DFilter* filt;
  const DMesh* mesh;
  const double* ebins;
  const int* fids;  // cell / material indices of cell and material filter bins
  double* value;
  // weight windows
  int ww_on, ww_mesh, ww_ne, ww_max_split;
  const double* ww_e;
  const double* ww_lower;
  const double* ww_upper;
  double ww_surv, ww_mlb, ww_cut;
  long long max_history_splits;
  // settings
  double energy_cutoff;
  double time_cutoff;  // neutron time cutoff in s (INFTY: none)
  int track_time;      // particle time is advanced (a time cutoff is set)
  int max_events;
  long long n_particles;
  long long master_seed;
  unsigned long long stride;
  // shared-memory copy of the per-event tables (tables_enter): byte offset
  // and 4-byte word count of each table, total bytes (0: not staged)
  int stage_off[9], stage_words[9];
  int stage_bytes;
};

// Particle bank, one slot per particle in flight.  The fields an event
// reads together sit together: slots are reached through a sorted queue, so
// the 32 lanes of a warp read 32 unrelated slots, and each field that lives
// in its own array costs a 32-byte memory sector per lane however few bytes
// it holds.  The hot fields are therefore packed into 16- and 32-byte
// records per slot (per level and slot for the coordinate levels: index
// l * cap + s), and reached through strided pointers so that every access
// reads db.f[k] as with plain arrays; the rest stay in arrays of their own.
// Counters that an event updates after it has stored a record (event count,
// collision count) and the particle id stay out of the records: reading a
// record back right after storing part of it waits for the store.
template<class T, int STRIDE>
struct Strided {
  T* p;  // the field in record 0
  __host__ __device__ __forceinline__ T& operator[](long long k) const
  {
    return *reinterpret_cast<T*>(reinterpret_cast<char*>(p) + k * STRIDE);
  }
};

struct alignas(32) BankDir {  // direction and energy
  double ux, uy, uz, E;
};
struct alignas(32) BankHot {  // random stream, weight, macroscopic total and absorption
  unsigned long long seed;
  double wgt, macro_t, macro_a;
};
struct alignas(16) BankMisc {  // coordinate depth, surface and materials
  int n_coord, surface, material, material_last;
};
struct alignas(32) BankPos {  // position at one coordinate level
  double x, y, z, pad;
};
struct alignas(32) BankIdx {  // cell, universe, lattice and lattice indices at one level
  int cell, univ, latt, lix, liy, liz, pad0, pad1;
};

template<class T>
using BField = Strided<T, 32>;
template<class T>
using BField16 = Strided<T, 16>;

struct DBank {
  long long cap;
  BankPos* pos;  // the records themselves, for whole-record loads and stores
  BankIdx* idx;
  BankDir* dir;
  BankHot* hot;
  BankMisc* misc;
  long long* id;
  BField<unsigned long long> seed;
  BField<double> E, wgt;
  double *wgt_born, *wgt_ww_born, *ww_factor;
  BField<double> ux, uy, uz;
  BField<double> rx, ry, rz;
  BField<int> cell, univ, latt, lix, liy, liz;
  BField16<int> n_coord;
  int *cell_last0, *cell_born;
  BField16<int> surface, material, material_last;
  BField<double> macro_t, macro_a;
  double* macro_nf;                  // macroscopic nu-fission (eigenvalue runs)
  double* time;                      // particle time in s (runs with a time cutoff)
  double *k_col, *k_abs, *k_tra;     // the history's k-effective scores (eigenvalue runs)
  int* n_progeny;                    // fission sites the history has banked
  int *bsurf, *blevel, *btrans;
  int *n_event, *n_collision, *n_split;
  int* sec_top;   // top of the slot's LIFO chain of banked secondaries
  int* sec_free;  // the slot's chain of pool entries already revived (reused first)
  int* n_total;  // events of the whole history (all revived secondaries)
};

struct DSecondary {
  double r[3], u[3], E, wgt, time;
  int surf, prev;
};

// A split particle waiting for a free slot of its own (split-to-slots mode):
// the parent's state at the split plus an independent tracking seed.
struct DSplitSite {
  double r[3], u[3];
  double E, wgt, wgt_born, wgt_ww_born, ww_factor, time;
  unsigned long long seed;
  long long id;
  int surf, n_split;
};

struct TraceRec {
  int32_t kind, cell, material, surface_or_nuclide, grid_hash, n_coord;
  double E, dist, wgt;
};

struct DCounters {
  int n_q, n_surf, n_coll, n_next, n_free;
  int refill_k, refill_free_base, pad0;
  long long refill_src, next_source, n_done;
  int n_sec, sec_cap;
  int error, n_lost;
  int iter, max_iter;
  double total_weight, leakage;
  unsigned long long n_events;
  long long lost_id;
  // event statistics for algorithmic-byte accounting, [0] queue kernels,
  // [1] tail kernel: xs events, xs recomputations, xs nuclide lookups, mesh
  // segments, collision nuclide lookups, surface events, collisions
  unsigned long long stat[2][7];
  unsigned long long n_refill;
  int more;  // set by the iteration epilogue when another iteration is needed
  int tail;  // 1 while the loop runs the remaining histories in k_tail
  int tail_threshold;  // queue length at or below which the tail phase starts
  unsigned long long longest;  // (events << 34) | particle id of the longest history
  // split-to-slots mode: ring of split particles waiting for a slot;
  // producers append at split_tail, the refill step consumes from split_head
  unsigned long long split_head, split_tail, refill_split_base;
  int refill_split;  // of this iteration's refill: how many come from the ring
  int split_cap;
  // eigenvalue runs: fission sites banked, bank overflow, and the
  // generation's collision, absorption and track-length k-effective sums
  unsigned long long n_fission;
  int fbank_full, pad1;
  double k_col, k_abs, k_tra;
};

// Source site of one history, sampled for the whole batch up front:
// position, direction, energy and the history's tracking-stream seed.
struct SourceSite {
  double r[3];
  double u[3];
  double E;
  unsigned long long tseed;
};

// Track records of one event iteration, written by the advance kernel at the
// event's queue position and scored by the track-length tally kernel
// (deferred scoring).  Structure of arrays over the bank capacity; inv_u only
// in FP32-table mode, mt/ma, mat and cell only when a tally needs them.
struct DTracks {
  double *r0x, *r0y, *r0z;  // start of the flight (level 0)
  double *ux, *uy, *uz;
  double *iux, *iuy, *iuz;  // 1 / u (FP32-table mode)
  double *d, *w, *E;        // flight length, weight (0: no record), pre-event energy
  double *mt, *ma;          // macroscopic total and absorption XS
  int* mat;                 // material
  int* cell;                // [MAXL][cap] cells of the levels, C_NONE past n_coord
};

struct DQueues {
  DTracks trk;           // deferred track records (trk.w null: tallies score inline)
  SourceSite* src_bank;  // [n_particles] or null (sites sampled at refill)
  double* src_time;      // the source sites' times (eigenvalue runs with a time cutoff), or null: 0
  long long src_n;
  int* q_in;
  int* q_surf;
  int* q_coll;
  int* q_tmp;
  int* key_tmp;  // sort key of each q_tmp entry, written with it (null: queue not sorted)
  int* free_list;
  int* hist;
  int* cursor;
  DSecondary* sec;
  DSplitSite* split;  // split-to-slots ring, or null
  // eigenvalue runs: the generation's fission bank (append order), its
  // capacity, the progeny count of each source index, and whether the source
  // bank already holds this generation's sites (every generation after the
  // first)
  DFissionSite* fbank;
  long long fbank_cap;
  int* progeny;
  int src_from_bank;
  int history;        // 1: history-based loop (slots are not recycled through the free list)
  DCounters* cnt;
  TraceRec* trace;
  int* trace_n;
  long long trace_hist;
  long long trace_first;  // first traced particle id
  int trace_cap;
  int trace_batch;  // batch whose histories are traced
  int batch;
  int sort_keys;
  int sort_sub_bits;  // sub-octave bits of the sort key (0 or 1)
};

// Defined here: this header is included by exactly one translation unit.
__constant__ DModel dm;
__constant__ DBank db;
__constant__ DQueues dq;

// ------------------------------------------------------ per-event tables
// The cell, surface, region-token, universe and per-material nuclide tables
// are read by every event.  Device code reaches them through the block's
// pointer table s_tabs, which each kernel sets at entry (tables_enter): to
// copies in dynamic shared memory when the stage_tables option is on and the
// launch provides room for all of them (dm.stage_bytes, at most
// OMC_STAGE_MAX_BYTES), else to the tables in global memory.
enum {
  STG_SURF, STG_CELL, STG_TOK, STG_UNIV_OFF, STG_UNIV_CELLS, STG_MAT_OFF, STG_MAT_NUC, STG_MAT_DENS,
  STG_MAT_DENS32, STG_N
};
static_assert(STG_N == sizeof(DModel::stage_off) / sizeof(int), "one staging slot per table");

#ifndef OMC_STAGE_MAX_BYTES
#define OMC_STAGE_MAX_BYTES 32768
#endif

struct Tabs {
  const DSurface* surf;
  const DCell* cell;
  const int* tok;
  const int* univ_off;
  const int* univ_cells;
  const int* mat_off;
  const int* mat_nuc;
  const double* mat_dens;
  const float* mat_dens32;
};

__shared__ Tabs s_tabs;
extern __shared__ __align__(16) unsigned char s_stage[];

__device__ __forceinline__ unsigned dynamic_smem_bytes()
{
  unsigned r;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
  return r;
}

__device__ __forceinline__ const void* stage_source(int k)
{
  switch (k) {
  case STG_SURF: return dm.surf;
  case STG_CELL: return dm.cell;
  case STG_TOK: return dm.tok;
  case STG_UNIV_OFF: return dm.univ_off;
  case STG_UNIV_CELLS: return dm.univ_cells;
  case STG_MAT_OFF: return dm.mat_off;
  case STG_MAT_NUC: return dm.mat_nuc;
  case STG_MAT_DENS: return dm.mat_dens;
  default: return dm.mat_dens32;
  }
}

// Sets s_tabs (copying the tables first when the launch's dynamic shared
// memory holds them).  Every thread of the block calls it, at kernel entry,
// before any thread can leave: it ends in a block barrier.
__device__ __forceinline__ void tables_enter()
{
  const bool stage = dm.stage_bytes > 0 && dynamic_smem_bytes() >= static_cast<unsigned>(dm.stage_bytes);
  if (stage) {
    for (int k = 0; k < STG_N; ++k) {
      const unsigned* src = static_cast<const unsigned*>(stage_source(k));
      unsigned* dst = reinterpret_cast<unsigned*>(s_stage + dm.stage_off[k]);
      for (int w = threadIdx.x; w < dm.stage_words[k]; w += blockDim.x) dst[w] = __ldg(src + w);
    }
  }
  if (threadIdx.x == 0) {
    if (stage) {
      s_tabs.surf = reinterpret_cast<const DSurface*>(s_stage + dm.stage_off[STG_SURF]);
      s_tabs.cell = reinterpret_cast<const DCell*>(s_stage + dm.stage_off[STG_CELL]);
      s_tabs.tok = reinterpret_cast<const int*>(s_stage + dm.stage_off[STG_TOK]);
      s_tabs.univ_off = reinterpret_cast<const int*>(s_stage + dm.stage_off[STG_UNIV_OFF]);
      s_tabs.univ_cells = reinterpret_cast<const int*>(s_stage + dm.stage_off[STG_UNIV_CELLS]);
      s_tabs.mat_off = reinterpret_cast<const int*>(s_stage + dm.stage_off[STG_MAT_OFF]);
      s_tabs.mat_nuc = reinterpret_cast<const int*>(s_stage + dm.stage_off[STG_MAT_NUC]);
      s_tabs.mat_dens = reinterpret_cast<const double*>(s_stage + dm.stage_off[STG_MAT_DENS]);
      s_tabs.mat_dens32 = reinterpret_cast<const float*>(s_stage + dm.stage_off[STG_MAT_DENS32]);
    } else {
      s_tabs.surf = dm.surf;
      s_tabs.cell = dm.cell;
      s_tabs.tok = dm.tok;
      s_tabs.univ_off = dm.univ_off;
      s_tabs.univ_cells = dm.univ_cells;
      s_tabs.mat_off = dm.mat_off;
      s_tabs.mat_nuc = dm.mat_nuc;
      s_tabs.mat_dens = dm.mat_dens;
      s_tabs.mat_dens32 = dm.mat_dens32;
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------- RNG
// src/random_lcg.cpp:32-44: one step of the generator and its output word
__host__ __device__ __forceinline__ unsigned long long prn_word(unsigned long long& s)
{
  s = PRN_MULT * s + PRN_ADD;
  unsigned long long word = ((s >> ((s >> 59u) + 5u)) ^ s) * 12605985483714917081ull;
  return (word >> 43u) ^ word;
}

// word x 2^-64 rounded to the nearest double (ldexp of the word converted to
// double, as the reference), built from the word's bits on the integer pipe
__device__ __forceinline__ double prn(unsigned long long& s)
{
  return fpi::u64_scaled_2m64(prn_word(s));
}

// The same generator step as prn, as an FP32 number in (0, 1): the top 23
// bits of the word, centred in their interval ((2k + 1) 2^-24 is exact in
// FP32), so that it is never 0 or 1 and its logarithm stays finite.
__device__ __forceinline__ float prn_f(unsigned long long& s)
{
  return __uint2float_rn(2u * static_cast<unsigned>(prn_word(s) >> 41) + 1u) * 0x1p-24f;
}

// src/random_lcg.cpp:91-120
__host__ __device__ inline unsigned long long future_seed(unsigned long long n, unsigned long long seed)
{
  unsigned long long g = PRN_MULT, c = PRN_ADD, g_new = 1, c_new = 0;
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

__device__ __forceinline__ double uniform_distribution(double a, double b, unsigned long long& s)
{
  return a + (b - a) * prn(s);
}

// src/math_functions.cpp:763-792 (phi sampled).  sin and cos of the sampled
// angle come from one sincos call (the device's own functions).
__device__ inline void rotate_angle(double& ux, double& uy, double& uz, double mu, unsigned long long& s)
{
  double phi_ = 2.0 * PI * prn(s);
  double sinphi, cosphi;
  sincos(phi_, &sinphi, &cosphi);
  // fmax(0, v) as the C library returns it (+0 for v <= 0), on the integer pipe
  const double va = 1. - mu * mu, vb = 1. - uz * uz;
  double a = sqrt(fpi::pos(va) ? va : 0.0);
  double b = sqrt(fpi::pos(vb) ? vb : 0.0);
  double x = ux, y = uy, z = uz;
  if (fpi::lt(1e-10, b)) {
    ux = mu * x + a * (x * z * cosphi - y * sinphi) / b;
    uy = mu * y + a * (y * z * cosphi + x * sinphi) / b;
    uz = mu * z - a * b * cosphi;
  } else {
    b = sqrt(1. - y * y);
    ux = mu * x + a * (-x * y * sinphi + z * cosphi) / b;
    uy = mu * y + a * b * sinphi;
    uz = mu * z - a * (y * z * sinphi + x * cosphi) / b;
  }
}

// rotate_angle in FP32 (FP32-table mode: the free-gas target direction and the
// centre-of-mass direction of an elastic scatter).  The
// perpendicular norm b is sqrt(ux^2 + uy^2) (sqrt(ux^2 + uz^2) in the second
// branch), which equals the reference's sqrt(1 - uz^2) for a unit vector
// and keeps FP32 accuracy when uz is near +-1, where 1 - uz^2 cancels.
__device__ inline void rotate_angle_f(float& ux, float& uy, float& uz, float mu, unsigned long long& s)
{
  float sinphi, cosphi;
  sincospif(2.0f * prn_f(s), &sinphi, &cosphi);
  const float a = sqrtf(fmaxf(0.f, 1.f - mu * mu));
  const float x = ux, y = uy, z = uz;
  float b = sqrtf(x * x + y * y);
  if (b > 1e-10f) {
    const float ib = 1.0f / b;
    ux = mu * x + a * (x * z * cosphi - y * sinphi) * ib;
    uy = mu * y + a * (y * z * cosphi + x * sinphi) * ib;
    uz = mu * z - a * b * cosphi;
  } else {
    b = sqrtf(x * x + z * z);
    const float ib = 1.0f / b;
    ux = mu * x + a * (-x * y * sinphi + z * cosphi) * ib;
    uy = mu * y + a * b * sinphi;
    uz = mu * z - a * (y * z * sinphi + x * cosphi) * ib;
  }
}

// src/random_dist.cpp:20-32
__device__ inline double maxwell_spectrum(double T, unsigned long long& s)
{
  double r1 = prn(s);
  double r2 = prn(s);
  double r3 = prn(s);
  double c = cos(PI / 2. * r3);
  return -T * (log(r1) + log(r2) * c * c);
}

// src/random_dist.cpp:34-43
__device__ inline double watt_spectrum(double a, double b, unsigned long long& s)
{
  double w = maxwell_spectrum(a, s);
  return w + 0.25 * a * a * b + uniform_distribution(-1., 1., s) * sqrt(a * a * b * w);
}

// Lower bound index on a sorted double range (include/openmc/search.h:14-20).
// Doubles of one sign order like their bit patterns; energies and bin edges
// here are non-negative, so the comparisons run on the integer pipe.
__device__ __forceinline__ int lower_bound_index_pos(const double* a, int lo, int hi, double v)
{
  // returns lower_bound(a+lo, a+hi, v) - (a+lo) - 1, or 0 when a[lo] == v
  if (__double_as_longlong(__ldg(a + lo)) == __double_as_longlong(v)) return 0;
  long long key = __double_as_longlong(v);
  int first = lo, count = hi - lo;
  while (count > 0) {
    int step = count >> 1;
    int it = first + step;
    if (__double_as_longlong(__ldg(a + it)) < key) {
      first = it + 1;
      count -= step + 1;
    } else {
      count = step;
    }
  }
  return first - lo - 1;
}

__device__ __forceinline__ int lower_bound_index_any(const double* a, int lo, int hi, double v)
{
  if (a[lo] == v) return 0;
  int first = lo, count = hi - lo;
  while (count > 0) {
    int step = count >> 1;
    int it = first + step;
    if (__ldg(a + it) < v) {
      first = it + 1;
      count -= step + 1;
    } else {
      count = step;
    }
  }
  return first - lo - 1;
}

// ------------------------------------------------------------- surfaces
// src/surface.cpp:116-130, 207-218, 399-442, 549-570
__device__ inline double surf_evaluate(const DSurface& s, double x, double y, double z)
{
  switch (s.type) {
  case 0: return x - s.c[0];
  case 1: return y - s.c[0];
  case 2: return z - s.c[0];
  case 3: { double a = fpi::sub(y, s.c[0]), b = fpi::sub(z, s.c[1]); return a * a + b * b - s.rr; }
  case 4: { double a = fpi::sub(x, s.c[0]), b = fpi::sub(z, s.c[1]); return a * a + b * b - s.rr; }
  case 5: { double a = fpi::sub(x, s.c[0]), b = fpi::sub(y, s.c[1]); return a * a + b * b - s.rr; }
  default: {
    double a = fpi::sub(x, s.c[0]), b = fpi::sub(y, s.c[1]), c = fpi::sub(z, s.c[2]);
    return a * a + b * b + c * c - s.rr;
  }
  }
}

// Comparisons run on the integer pipe (fp64_int.cuh) with the IEEE results.
// inv_u_i: 1 / u_i in FP32-table mode (a product replaces the quotient),
// 0 for the reference's division.
__device__ inline double plane_distance(double r_i, double u_i, bool coincident, double offset, double inv_u_i = 0.0)
{
  const double f = offset - r_i;
  if (coincident || fpi::abs_lt(f, FP_COINCIDENT) || fpi::zero(u_i)) return INFTY;
  // f / u_i < 0 exactly when the signs differ (f and u_i are non-zero here,
  // |f| >= 1e-12 and |u_i| <= 1, so the quotient is never a zero): skip the
  // division then; otherwise the quotient is positive and the reference's
  // d < 0 test never holds
  if ((fpi::bits(f) ^ fpi::bits(u_i)) < 0) return INFTY;
  return fpi::zero(inv_u_i) ? f / u_i : f * inv_u_i;
}

// Square root for FP32-table mode geometry: the FP32 root of q refined by one
// Newton step in FP64, y0 + (q - y0^2) / (2 y0), with 1 / (2 y0) taken in
// FP32 (the correction is of order 1e-7 y0, so its own FP32 error is of
// order 1e-14 of the root; the step leaves a relative error of order 1e-14
// against 1e-16 for the FP64 root, far inside the geometry's 1e-14 and 1e-8
// cm tolerances), two FP64 operations in place of the FP64 square root.
// Outside [1e-30, 1e30] (never for centimetre geometry) the FP64 root.
__device__ __forceinline__ double sqrt_refined(double q)
{
  if (!(fpi::bits(q) >= fpi::bits(1e-30) && fpi::bits(q) <= fpi::bits(1e30))) return sqrt(q);
  const float y0f = sqrtf(fpi::to_float(q));
  const double y0 = fpi::to_double(y0f);
  return fma(fma(-y0, y0, q), fpi::to_double(0.5f / y0f), y0);
}

// inv_a: 1 / (1 - u1^2) in FP32-table mode (products replace the quotients,
// sqrt_refined the root), 0 for the reference's divisions and root.
__device__ inline double cylinder_distance(double u1, double r2_, double u2, double r3_, double u3,
  bool coincident, double offset1, double offset2, double radius, double inv_a = 0.0)
{
  const double a = 1.0 - u1 * u1;
  if (fpi::zero(a)) return INFTY;
  const double r2 = fpi::sub(r2_, offset1);
  const double r3 = fpi::sub(r3_, offset2);
  const double k = r2 * u2 + r3 * u3;
  const double c = r2 * r2 + r3 * r3 - radius;  // radius: the squared radius
  const double quad = k * k - a * c;
  const bool prod = !fpi::zero(inv_a);
  if (fpi::neg(quad)) {
    return INFTY;
  } else if (coincident || fpi::abs_lt(c, FP_COINCIDENT)) {
    if (fpi::nonneg(k)) return INFTY;
    return prod ? (-k + sqrt_refined(quad)) * inv_a : (-k + sqrt(quad)) / a;
  } else if (fpi::neg(c)) {
    return prod ? (-k + sqrt_refined(quad)) * inv_a : (-k + sqrt(quad)) / a;
  } else {
    const double d = prod ? (-k - sqrt_refined(quad)) * inv_a : (-k - sqrt(quad)) / a;
    if (fpi::neg(d)) return INFTY;
    return d;
  }
}

__device__ inline double sphere_distance(const DSurface& s, double x_, double y_, double z_, double ux,
  double uy, double uz, bool coincident)
{
  const double x = fpi::sub(x_, s.c[0]);
  const double y = fpi::sub(y_, s.c[1]);
  const double z = fpi::sub(z_, s.c[2]);
  const double k = x * ux + y * uy + z * uz;
  const double c = x * x + y * y + z * z - s.rr;
  const double quad = k * k - c;
  if (fpi::neg(quad)) {
    return INFTY;
  } else if (coincident || fpi::abs_lt(c, FP_COINCIDENT)) {
    if (fpi::nonneg(k)) return INFTY;
    return -k + sqrt(quad);
  } else if (fpi::neg(c)) {
    return -k + sqrt(quad);
  } else {
    const double d = -k - sqrt(quad);
    if (fpi::neg(d)) return INFTY;
    return d;
  }
}

// inv_u (FP32-table mode): 1/ux, 1/uy, 1/uz and 1/(1 - uz^2) of the flight
__device__ inline double surf_distance(const DSurface& s, double x, double y, double z, double ux,
  double uy, double uz, bool coincident, const double* inv_u = nullptr)
{
  switch (s.type) {
  case 0: return plane_distance(x, ux, coincident, s.c[0], inv_u ? inv_u[0] : 0.0);
  case 1: return plane_distance(y, uy, coincident, s.c[0], inv_u ? inv_u[1] : 0.0);
  case 2: return plane_distance(z, uz, coincident, s.c[0], inv_u ? inv_u[2] : 0.0);
  case 3: return cylinder_distance(ux, y, uy, z, uz, coincident, s.c[0], s.c[1], s.rr);
  case 4: return cylinder_distance(uy, x, ux, z, uz, coincident, s.c[0], s.c[1], s.rr);
  case 5: return cylinder_distance(uz, x, ux, y, uy, coincident, s.c[0], s.c[1], s.rr, inv_u ? inv_u[3] : 0.0);
  default: return sphere_distance(s, x, y, z, ux, uy, uz, coincident);
  }
}

__device__ inline void surf_normal(const DSurface& s, double x, double y, double z, double& nx, double& ny, double& nz)
{
  switch (s.type) {
  case 0: nx = 1.; ny = 0.; nz = 0.; return;
  case 1: nx = 0.; ny = 1.; nz = 0.; return;
  case 2: nx = 0.; ny = 0.; nz = 1.; return;
  case 3: nx = 0.0; ny = 2.0 * (y - s.c[0]); nz = 2.0 * (z - s.c[1]); return;
  case 4: nx = 2.0 * (x - s.c[0]); ny = 0.0; nz = 2.0 * (z - s.c[1]); return;
  case 5: nx = 2.0 * (x - s.c[0]); ny = 2.0 * (y - s.c[1]); nz = 0.0; return;
  default: nx = 2.0 * (x - s.c[0]); ny = 2.0 * (y - s.c[1]); nz = 2.0 * (z - s.c[2]); return;
  }
}

__device__ inline bool surf_sense(const DSurface& s, double x, double y, double z, double ux, double uy, double uz)
{
  const double f = surf_evaluate(s, x, y, z);
  if (fpi::abs_lt(f, FP_COINCIDENT)) {
    double nx, ny, nz;
    surf_normal(s, x, y, z, nx, ny, nz);
    return fpi::pos(ux * nx + uy * ny + uz * nz);
  }
  return fpi::pos(f);
}

// src/cell.cpp:951-969 simple regions; postfix evaluation for complex ones
__device__ inline bool cell_contains(const DCell& c, double x, double y, double z, double ux, double uy,
  double uz, int on_surface)
{
  const int* t = s_tabs.tok + c.tok_off;
  if (c.simple) {
    for (int k = 0; k < c.tok_len; ++k) {
      int token = t[k];
      if (token == on_surface) {
      } else if (-token == on_surface) {
        return false;
      } else {
        bool sense = surf_sense(s_tabs.surf[abs(token) - 1], x, y, z, ux, uy, uz);
        if (sense != (token > 0)) return false;
      }
    }
    return true;
  }
  unsigned stack = 0;  // bit stack, depth <= 32
  int sp = 0;
  for (int k = 0; k < c.tok_len; ++k) {
    int token = t[k];
    if (token < 2147483643) {  // OP_UNION
      bool v;
      if (token == on_surface) v = true;
      else if (-token == on_surface) v = false;
      else v = (surf_sense(s_tabs.surf[abs(token) - 1], x, y, z, ux, uy, uz) == (token > 0));
      stack = (stack & ~(1u << sp)) | (unsigned(v) << sp);
      ++sp;
    } else if (token == 2147483645) {  // OP_COMPLEMENT
      stack ^= 1u << (sp - 1);
    } else {
      bool b = (stack >> (sp - 1)) & 1u;
      bool a = (stack >> (sp - 2)) & 1u;
      bool r = (token == 2147483644) ? (a && b) : (a || b);  // INTERSECTION / UNION
      --sp;
      stack = (stack & ~(1u << (sp - 1))) | (unsigned(r) << (sp - 1));
    }
  }
  return sp > 0 ? (stack & 1u) : true;
}

// src/cell.cpp:910-936.  `bound` lets the caller skip axis-aligned planes
// whose perpendicular distance |f| (a lower bound of the distance along any
// direction) already exceeds it; skipped planes count as no crossing.  With
// bound = INFTY this is exactly the reference loop.
__device__ inline void region_distance(const DCell& c, double x, double y, double z, double ux, double uy,
  double uz, int on_surface, double& min_dist, int& i_surf, double bound = INFTY, const double* inv_u = nullptr)
{
  min_dist = INFTY;
  i_surf = 2147483647;
  const int* t = s_tabs.tok + c.tok_off;
  for (int k = 0; k < c.tok_len; ++k) {
    int token = t[k];
    if (token >= 2147483643) continue;
    const DSurface& sf = s_tabs.surf[abs(token) - 1];
    if (sf.type <= 2) {
      double r_i = sf.type == 0 ? x : (sf.type == 1 ? y : z);
      if (fpi::abs_gt(sf.c[0] - r_i, bound)) continue;
    }
    bool coincident = abs(token) == abs(on_surface);
    double d = surf_distance(sf, x, y, z, ux, uy, uz, coincident, inv_u);
    if (fpi::lt(d, min_dist)) {
      // the first candidate against INFTY always passes: INFTY - d rounds
      // to INFTY, which exceeds FP_PRECISION x INFTY
      if (fpi::bits(min_dist) == fpi::bits(INFTY) || fpi::le(FP_PRECISION * min_dist, min_dist - d)) {
        min_dist = d;
        i_surf = -token;
      }
    }
  }
}

// ------------------------------------------------------------- lattices
// src/lattice.cpp:252-306
// inv_u: 1/u per axis (FP32-table mode: the quotients become products,
// still FP64 but rounded twice), or null for the reference's divisions.
__device__ inline double lattice_distance(const DLattice& lat, double x, double y, double z, double ux,
  double uy, double uz, int& trans, const double* inv_u = nullptr)
{
  // x0 - x is exactly -(x - x0), so |x - x0| is read from the one difference
  const double x0 = copysign(lat.half[0], ux);
  const double y0 = copysign(lat.half[1], uy);
  double d = INFTY;
  trans = 13;  // encoded (tx+1) + 3(ty+1) + 9(tz+1); 13 == no translation
  const double fx = x0 - x;
  if (fpi::abs_gt(fx, FP_PRECISION) && !fpi::zero(ux)) {
    d = inv_u ? fx * inv_u[0] : fx / ux;
    trans = fpi::pos(ux) ? 14 : 12;
  }
  const double fy = y0 - y;
  if (fpi::abs_gt(fy, FP_PRECISION) && !fpi::zero(uy)) {
    double this_d = inv_u ? fy * inv_u[1] : fy / uy;
    if (fpi::lt(this_d, d)) {
      d = this_d;
      trans = fpi::pos(uy) ? 16 : 10;
    }
  }
  if (lat.is3d) {
    const double z0 = copysign(lat.half[2], uz);
    const double fz = z0 - z;
    if (fpi::abs_gt(fz, FP_PRECISION) && !fpi::zero(uz)) {
      double this_d = inv_u ? fz * inv_u[2] : fz / uz;
      if (fpi::lt(this_d, d)) {
        d = this_d;
        trans = fpi::pos(uz) ? 22 : 4;
      }
    }
  }
  return d;
}

// src/lattice.cpp:310-342
__device__ inline void lattice_get_indices(const DLattice& lat, double x, double y, double z, double ux,
  double uy, double uz, int* res)
{
  double ix_ = (x - lat.ll[0]) / lat.pitch[0];
  long long ix_close = llround(ix_);
  if (fabs(ix_ - ix_close) < FP_COINCIDENT) res[0] = (ux > 0) ? ix_close : ix_close - 1;
  else res[0] = static_cast<int>(floor(ix_));
  double iy_ = (y - lat.ll[1]) / lat.pitch[1];
  long long iy_close = llround(iy_);
  if (fabs(iy_ - iy_close) < FP_COINCIDENT) res[1] = (uy > 0) ? iy_close : iy_close - 1;
  else res[1] = static_cast<int>(floor(iy_));
  res[2] = 0;
  if (lat.is3d) {
    double iz_ = (z - lat.ll[2]) / lat.pitch[2];
    long long iz_close = llround(iz_);
    if (fabs(iz_ - iz_close) < FP_COINCIDENT) res[2] = (uz > 0) ? iz_close : iz_close - 1;
    else res[2] = static_cast<int>(floor(iz_));
  }
}

// src/lattice.cpp:352-361
// (i + 0.5 formed on the integer pipe, exactly)
__device__ inline void lattice_local_position(const DLattice& lat, double& x, double& y, double& z, const int* i)
{
  x -= (lat.ll[0] + fpi::half_odd(i[0]) * lat.pitch[0]);
  y -= (lat.ll[1] + fpi::half_odd(i[1]) * lat.pitch[1]);
  if (lat.is3d) z -= (lat.ll[2] + fpi::half_odd(i[2]) * lat.pitch[2]);
}

__device__ __forceinline__ bool lattice_valid(const DLattice& lat, const int* i)
{
  return i[0] >= 0 && i[0] < lat.n[0] && i[1] >= 0 && i[1] < lat.n[1] && i[2] >= 0 && i[2] < lat.n[2];
}

// ------------------------------------------------------- particle geometry
// Register copy of a particle's coordinate levels.
struct Geo {
  double r[MAXL][3];
  double u[3];
  double E;  // loaded with the direction (geo_store does not write it)
  int cell[MAXL], univ[MAXL], lat[MAXL], li[MAXL][3];
  int n_coord;
  int surface;
  int material, material_last;
};

// Per-level arrays of a Geo are only ever indexed by compile-time levels
// (loops over levels are unrolled up to MAXL with a run-time guard, and a
// level known only at run time is read through lvl_get), so that the
// compiler can keep them in registers instead of thread-local memory.
template<class T>
__device__ __forceinline__ T lvl_get(const T (&a)[MAXL], int l)
{
  T v = a[0];
#pragma unroll
  for (int k = 1; k < MAXL; ++k)
    if (l == k) v = a[k];
  return v;
}

__device__ inline void geo_load(Geo& g, long long s)
{
  const long long cap = db.cap;
  const BankMisc mi = db.misc[s];
  const BankDir d = db.dir[s];
  g.n_coord = mi.n_coord;
  g.u[0] = d.ux;
  g.u[1] = d.uy;
  g.u[2] = d.uz;
  g.E = d.E;
#pragma unroll
  for (int l = 0; l < MAXL; ++l) {
    if (l >= g.n_coord) break;
    long long k = l * cap + s;
    const BankPos p = db.pos[k];
    const BankIdx x = db.idx[k];
    g.r[l][0] = p.x;
    g.r[l][1] = p.y;
    g.r[l][2] = p.z;
    g.cell[l] = x.cell;
    g.univ[l] = x.univ;
    g.lat[l] = x.latt;
    g.li[l][0] = x.lix;
    g.li[l][1] = x.liy;
    g.li[l][2] = x.liz;
  }
  g.surface = mi.surface;
  g.material = mi.material;
  g.material_last = mi.material_last;
}

__device__ inline void geo_store(const Geo& g, long long s)
{
  const long long cap = db.cap;
  db.n_coord[s] = g.n_coord;
  db.ux[s] = g.u[0];
  db.uy[s] = g.u[1];
  db.uz[s] = g.u[2];
#pragma unroll
  for (int l = 0; l < MAXL; ++l) {
    if (l >= g.n_coord) break;
    long long k = l * cap + s;
    BankPos p;
    p.x = g.r[l][0];
    p.y = g.r[l][1];
    p.z = g.r[l][2];
    p.pad = 0.0;
    db.pos[k] = p;
    BankIdx x;
    x.cell = g.cell[l];
    x.univ = g.univ[l];
    x.latt = g.lat[l];
    x.lix = g.li[l][0];
    x.liy = g.li[l][1];
    x.liz = g.li[l][2];
    x.pad0 = x.pad1 = 0;
    db.idx[k] = x;
  }
  db.surface[s] = g.surface;
  db.material[s] = g.material;
  db.material_last[s] = g.material_last;
}

// New direction of slot s
__device__ __forceinline__ void set_direction(long long s, double ux, double uy, double uz)
{
  db.ux[s] = ux;
  db.uy[s] = uy;
  db.uz[s] = uz;
}

__device__ __forceinline__ void coord_reset(Geo& g, int l)
{
  g.cell[l] = C_NONE;
  g.univ[l] = C_NONE;
  g.lat[l] = C_NONE;
  g.li[l][0] = g.li[l][1] = g.li[l][2] = 0;
}

// src/universe.cpp:40-59 at coordinate level lvl (a compile-time level
// wherever this is inlined)
__device__ __forceinline__ bool universe_find_cell(Geo& g, const int lvl)
{
  int u = g.univ[lvl];
  int a = s_tabs.univ_off[u], b = s_tabs.univ_off[u + 1];
  for (int k = a; k < b; ++k) {
    int ic = s_tabs.univ_cells[k];
    const DCell& c = s_tabs.cell[ic];
    if (c.universe != u) continue;
    if (cell_contains(c, g.r[lvl][0], g.r[lvl][1], g.r[lvl][2], g.u[0], g.u[1], g.u[2], g.surface)) {
      g.cell[lvl] = ic;
      return true;
    }
  }
  return false;
}

// src/geometry.cpp:102-252 (exhaustive branch; neighbour lists are an
// ordering optimisation with the same result for non-overlapping cells)
__device__ inline bool find_cell_inner(Geo& g, bool& lost_outer)
{
  const int start = g.n_coord - 1;
#pragma unroll
  for (int lvl = 0; lvl < MAXL; ++lvl) {
    if (lvl < start) continue;
    g.n_coord = lvl + 1;
    if (!universe_find_cell(g, lvl)) return false;
    const DCell& c = s_tabs.cell[g.cell[lvl]];
    if (c.fill_type == 0) {
      g.material_last = g.material;
      g.material = c.fill;
      return true;
    }
    if (g.n_coord >= dm.n_coord_levels || lvl + 1 >= MAXL) return false;
    const int nl = lvl + 1 < MAXL ? lvl + 1 : lvl;  // == lvl + 1 on every path that reaches it
    g.r[nl][0] = fpi::sub(g.r[lvl][0], c.tr[0]);
    g.r[nl][1] = fpi::sub(g.r[lvl][1], c.tr[1]);
    g.r[nl][2] = fpi::sub(g.r[lvl][2], c.tr[2]);
    if (c.fill_type == 1) {
      g.univ[nl] = c.fill;
      g.lat[nl] = C_NONE;
    } else {
      const DLattice& lat = dm.lat[c.fill];
      lattice_get_indices(lat, g.r[nl][0], g.r[nl][1], g.r[nl][2], g.u[0], g.u[1], g.u[2], g.li[nl]);
      lattice_local_position(lat, g.r[nl][0], g.r[nl][1], g.r[nl][2], g.li[nl]);
      g.lat[nl] = c.fill;
      if (lattice_valid(lat, g.li[nl])) {
        g.univ[nl] = dm.lat_univ[lat.univ_off + lat.n[0] * lat.n[1] * g.li[nl][2] + lat.n[0] * g.li[nl][1] + g.li[nl][0]];
      } else if (lat.outer != -1) {
        g.univ[nl] = lat.outer;
      } else {
        lost_outer = true;
        return false;
      }
    }
    g.cell[nl] = C_NONE;
  }
  return false;
}

// src/geometry.cpp:284-298
__device__ inline bool exhaustive_find_cell(Geo& g, bool& lost_outer)
{
  if (lvl_get(g.univ, g.n_coord - 1) == C_NONE) {
    g.univ[0] = dm.root_univ;
    g.n_coord = 1;
  }
  return find_cell_inner(g, lost_outer);
}

// (t / d >= FP_REL_PRECISION) with the quotient rounded as the reference
// rounds it.  For a finite d >= 2^-959, t at or above d x 1e-5 (1 + 2^-40),
// or at or below d x 1e-5 (1 - 2^-40), each product rounded once, settles
// the rounded quotient on its side of the threshold (the margin is far
// above the 2^-53 relative error of the product and of the quotient), so
// the FP64 division runs only for t within that margin, or for d not
// positive and finite.
__device__ __forceinline__ bool rel_gap_at_least(double t, double d)
{
  // d in [2^-959, inf): the products stay normal doubles
  if (fpi::bits(d) >= 0x0400000000000000LL && fpi::bits(d) < fpi::EXP_INF) {
    if (fpi::le(d * 1.0000000000009096e-05, t)) return true;   // 1e-5 (1 + 2^-40)
    if (fpi::le(t, d * 9.999999999990905e-06)) return false;   // 1e-5 (1 - 2^-40)
  }
  return t / d >= FP_REL_PRECISION;
}

// src/geometry.cpp:361-453.  The levels below the root are evaluated first;
// the candidate distance D of level 1 bounds the root level: the reference
// replaces any root distance above D (1 + 1e-4) by D at level 1 (its
// FP_REL_PRECISION test is 1e-5), so root planes whose perpendicular
// distance exceeds that bound are skipped, and a root level whose every
// surface was skipped enters the level loop as INFINITY.  The returned
// boundary is the reference's.
__device__ inline void distance_to_boundary(const Geo& g, double& dist, int& surface, int& level,
  int& trans, bool& neg_lat, const double* inv_u = nullptr)
{
  const double INF = __longlong_as_double(0x7ff0000000000000LL);  // INFINITY
  double ds[MAXL], dl[MAXL];
  int ss[MAXL], tt[MAXL];
  double bound = INF;
#pragma unroll
  for (int i = MAXL - 1; i >= 0; --i) {
    if (i >= g.n_coord) continue;
    const DCell& c = s_tabs.cell[g.cell[i]];
    const double* r = g.r[i];
    double b = (i == 0 && g.n_coord > 1) ? bound : INFTY;
    region_distance(c, r[0], r[1], r[2], g.u[0], g.u[1], g.u[2], g.surface, ds[i], ss[i], b, inv_u);
    if (i == 0 && g.n_coord > 1 && ss[i] == 2147483647) ds[i] = INF;  // every root surface bounded away
    dl[i] = INF;
    tt[i] = 13;
    if (g.lat[i] != C_NONE) {
      dl[i] = lattice_distance(dm.lat[g.lat[i]], r[0], r[1], r[2], g.u[0], g.u[1], g.u[2], tt[i], inv_u);
      if (fpi::neg(dl[i])) neg_lat = true;
    }
    if (i == 1) {
      // candidate of the level directly below the root: any root distance
      // above cand (1 + 1e-4) loses to it in the level loop below
      double cand = fpi::lt(ds[i], dl[i] - FP_COINCIDENT) ? ds[i] : dl[i];
      bound = cand * (1.0 + 1e-4);
    }
  }
  dist = INF;
  surface = SURFACE_NONE;
  level = 0;
  trans = 13;
#pragma unroll
  for (int i = 0; i < MAXL; i++) {
    if (i >= g.n_coord) break;
    const DCell& c = s_tabs.cell[g.cell[i]];
    const double* r = g.r[i];
    double d_surf = ds[i];
    double d_lat = dl[i];
    double& d = dist;
    if (fpi::lt(d_surf, d_lat - FP_COINCIDENT)) {
      if (fpi::bits(d) == fpi::bits(INF) || rel_gap_at_least(d - d_surf, d)) {
        d = d_surf;
        if (c.simple || fpi::bits(d) == fpi::bits(INFTY)) {
          surface = ss[i];
        } else {
          double hx = r[0] + d_surf * g.u[0];
          double hy = r[1] + d_surf * g.u[1];
          double hz = r[2] + d_surf * g.u[2];
          double nx, ny, nz;
          surf_normal(s_tabs.surf[abs(ss[i]) - 1], hx, hy, hz, nx, ny, nz);
          surface = fpi::pos(g.u[0] * nx + g.u[1] * ny + g.u[2] * nz) ? abs(ss[i]) : -abs(ss[i]);
        }
        trans = 13;
        level = i + 1;
      }
    } else {
      if (fpi::bits(d) == fpi::bits(INF) || rel_gap_at_least(d - d_lat, d)) {
        d = d_lat;
        surface = SURFACE_NONE;
        trans = tt[i];
        level = i + 1;
      }
    }
  }
}

// --------------------------------------------------------- cross sections
// Per-nuclide lookup: src/nuclide.cpp:724-775 (single temperature).
struct Micro {
  double total, absorption;
  int i_grid;
  double f;
  double fission, nu_fission;  // interpolated only when asked for (eigenvalue runs)
};

// Locates the grid interval of E and returns its index and bracketing
// energies e0 < e1 (duplicate points skipped as the reference does).
// Energies are non-negative doubles, which order (and compare equal) like
// their bit patterns: the comparisons run on the integer pipe.
__device__ __forceinline__ int nuclide_grid(int nuc, int i_log, double E, double& e0_out, double& e1_out)
{
  const long long off = dm.nuc_off[nuc];
  const int G = static_cast<int>(dm.nuc_off[nuc + 1] - off);
  const double* e = dm.energy + off;
  const long long kE = __double_as_longlong(E);
  int i_grid;
  if (kE < __double_as_longlong(__ldg(e))) {
    i_grid = 0;
  } else if (kE > __double_as_longlong(__ldg(e + G - 1))) {
    i_grid = G - 2;
  } else {
    const int* gi = dm.grid_index + static_cast<long long>(nuc) * (dm.M + 1);
    int i_low = __ldg(gi + i_log);
    int i_high = __ldg(gi + i_log + 1) + 1;
    i_grid = i_low + lower_bound_index_pos(e, i_low, i_high, E);
  }
  double e0 = __ldg(e + i_grid), e1 = __ldg(e + i_grid + 1);
  if (__double_as_longlong(e0) == __double_as_longlong(e1)) {
    ++i_grid;
    e0 = e1;
    e1 = __ldg(e + i_grid + 1);
  }
  e0_out = e0;
  e1_out = e1;
  return i_grid;
}

// one FP64 row as two 16-byte read-only loads
__device__ __forceinline__ XsRow64 ldg_row(const XsRow64* p)
{
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldg(q);
  const double2 b = __ldg(q + 1);
  return XsRow64 {a.x, a.y, b.x, b.y};
}

// fiss: also interpolate the fission and nu-fission columns (the same two
// rows, src/nuclide.cpp:760-775)
__device__ __forceinline__ Micro micro_xs64(int nuc, int i_log, double E, bool fiss = false)
{
  Micro m;
  double e0, e1;
  m.i_grid = nuclide_grid(nuc, i_log, E, e0, e1);
  m.f = (E - e0) / (e1 - e0);
  const XsRow64* xs = dm.xs64 + dm.nuc_off[nuc];
  const XsRow64 a = ldg_row(xs + m.i_grid);
  const XsRow64 b = ldg_row(xs + m.i_grid + 1);
  m.total = (1.0 - m.f) * a.total + m.f * b.total;
  m.absorption = (1.0 - m.f) * a.absorption + m.f * b.absorption;
  m.fission = m.nu_fission = 0.0;
  if (fiss) {
    m.fission = (1.0 - m.f) * a.fission + m.f * b.fission;
    m.nu_fission = (1.0 - m.f) * a.nu_fission + m.f * b.nu_fission;
  }
  return m;
}

// FP32 tables: the grid search stays FP64 (E against FP64 grid energies);
// the interpolation factor is the FP64 difference E - e0 rounded to FP32
// times the interval's reciprocal width stored (rounded to FP32) in the
// row's last slot, and the interpolation is written a + f (b - a), which
// stays accurate when f leaves [0, 1] (energies below the first or above the
// last grid point extrapolate); (1 - f) a + f b cancels catastrophically in
// FP32 there.
// (the row's z is nu-fission; nf receives it interpolated when not null)
__device__ __forceinline__ void micro_xs32(int nuc, int i_log, double E, float& t, float& a_out, int& i_grid, float& f32,
  float* nf = nullptr)
{
  double e0, e1;
  i_grid = nuclide_grid(nuc, i_log, E, e0, e1);
  const float4* xs = dm.xs32 + dm.nuc_off[nuc];
  float4 a = __ldg(xs + i_grid);
  float4 b = __ldg(xs + i_grid + 1);
  f32 = fpi::to_float(E - e0) * a.w;
  t = a.x + f32 * (b.x - a.x);
  a_out = a.y + f32 * (b.y - a.y);
  if (nf) *nf = a.z + f32 * (b.z - a.z);
}

// Hash bin of E (src/material.cpp:833-834), clamped to [0, M-1]: the
// reference reads grid_index[M+1] past the end of the table for E equal to
// the grid maximum (and a negative bin below the minimum); the clamp keeps
// the search window inside the table and the located grid index unchanged.
// The bin is first formed in FP32, (logf(E) - log e_min) / spacing: E
// rounded to FP32 (6e-8 relative), logf within 1 ulp and the two rounded
// constants put it within 2e-3 bins of the exact quotient, so when it lies
// more than 1/64 bin from an integer its floor is the reference's FP64
// result; otherwise (and for non-finite values) the FP64 expression decides.
// The returned bin is always the FP64 expression's.
__device__ __forceinline__ int log_union_index(double E)
{
  const float q = (logf(fpi::to_float(E)) - dm.log_emin32) * dm.inv_spacing32;
  const float fl = floorf(q);
  const float fr = q - fl;
  int i;
  if (fr > 0.015625f && fr < 0.984375f && fabsf(q) < 1.0e7f) i = static_cast<int>(fl);
  else i = static_cast<int>(log(E / dm.e_min) / dm.log_spacing);
  return i < 0 ? 0 : (i > dm.M - 1 ? dm.M - 1 : i);
}

// src/material.cpp:829-901.  Returns the grid-index hash of the material's
// nuclides (h = 31 h + i_grid) for per-history trace comparison.  nf (an
// eigenvalue run) receives the macroscopic nu-fission cross section.
__device__ inline uint32_t material_xs(int mat, double E, double& tot, double& abs_, double* nf = nullptr)
{
  int i_log = log_union_index(E);
  int a = s_tabs.mat_off[mat], b = s_tabs.mat_off[mat + 1];
  uint32_t h = 0;
  const bool fiss = nf != nullptr;
  if (!dm.xs_fp32) {
    double t = 0.0, ab = 0.0, nuf = 0.0;
    for (int k = a; k < b; ++k) {
      int nuc = s_tabs.mat_nuc[k];
      Micro m = micro_xs64(nuc, i_log, E, fiss);
      h = h * 31u + static_cast<uint32_t>(m.i_grid);
      double dens = s_tabs.mat_dens[k];
      t += dens * m.total;
      ab += dens * m.absorption;
      if (fiss) nuf += dens * m.nu_fission;
    }
    tot = t;
    abs_ = ab;
    if (fiss) *nf = nuf;
  } else {
    float t = 0.0f, ab = 0.0f, nuf = 0.0f;
    for (int k = a; k < b; ++k) {
      int nuc = s_tabs.mat_nuc[k];
      float mt, ma, f32, mnf = 0.0f;
      int ig;
      micro_xs32(nuc, i_log, E, mt, ma, ig, f32, fiss ? &mnf : nullptr);
      h = h * 31u + static_cast<uint32_t>(ig);
      float dens = s_tabs.mat_dens32[k];
      t += dens * mt;
      ab += dens * ma;
      nuf += dens * mnf;
    }
    tot = fpi::to_double(t);
    abs_ = fpi::to_double(ab);
    if (fiss) *nf = fpi::to_double(nuf);
  }
  return h;
}

}  // namespace OMC_NS
}  // namespace omc
