// Host interface of the GPU transport layer (implemented in transport.cu).
#pragma once

#include "host_model.h"

namespace omc {

// device error flags (bitwise OR in the batch counters)
constexpr int ERR_LOST = 1, ERR_SECONDARY_OVERFLOW = 2, ERR_NO_NUCLIDE = 4,
              ERR_ITERATIONS = 8, ERR_REJECTION = 16, ERR_TRACE = 32, ERR_BANK = 64;

struct GpuSim;

struct GpuOptions {
  long long in_flight = 0;      // particle slots in HBM (0: min(n_particles, 2^19))
  long long secondary_cap = 0;  // secondary-site pool entries (0: automatic)
  bool xs_fp32 = false;         // FP32 cross-section tables and interpolation
  bool sort = true;             // sort the cross-section queue by (material, energy)
  long long tail_threshold = -1;  // queue length for the history-based tail (-1: default)
  int fuse = 3;                 // bit 0: cross-section event, bit 1: surface crossing, inside the advance kernel
  int split_slots = 0;          // split particles start in free slots with their own seeds
  int max_levels = 0;           // coordinate depth of the kernels (0: the model's, rounded up to 2 or 4)
  int stage_tables = 0;         // copy the cell/surface/material tables into shared memory per block
  int contract = 1;             // FP32-table mode: run the build with FP64 multiply-adds fused
  int defer_tally = 1;          // track-length tallies scored by their own kernel from track records
};

// One MAGIC weight-window update (WeightWindows::update_weights,
// src/weight_windows.cpp:502-755) from a flux tally's accumulated sums.
struct MagicArgs {
  int tally = 0;              // tally index
  int score = 0;              // position of the flux score among the tally's scores
  int n_scores = 1;
  long long stride_mesh = 1;  // filter-bin stride of the mesh filter
  long long stride_energy = -1;  // of the energy filter, -1: none
  int e_bins = 1;
  long long mesh_bins = 1;
  int n = 1;                  // realizations
  double volume = 1.0;        // of one mesh element
  int rel_err = 0;            // 1: bounds from 1 / relative error, 0: from the mean
  double threshold = 1.0, ratio = 5.0;
};

// Bookkeeping of one eigenvalue generation, read after its transport.
struct GenerationStats {
  long long fission_sites = 0;
  double k_col = 0, k_abs = 0, k_tra = 0;  // the generation's k-effective sums
  double total_weight = 0;
};

struct BatchStats {
  float ms = 0;
  int error = 0;
  int n_lost = 0;
  long long lost_id = 0;
  long long n_done = 0;
  int iterations = 0;
  double total_weight = 0;
  double leakage = 0;
  unsigned long long n_events = 0;
  int n_secondaries = 0;
  long long longest_events = 0, longest_id = 0;  // longest history of the batch
  // [queue, tail] x [xs events, xs recomputations, xs nuclide lookups, mesh
  // segments, collision nuclide lookups, surface events, collisions]
  unsigned long long stat[2][7] = {{0, 0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0, 0}};
  // per-kernel device milliseconds from a profiled batch:
  // xs, advance, surface, collision, tail, refill, sort, other, track-length tally
  float kernel_ms[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
};

// The interface below is implemented three times: transport.cu built for at
// most 2 and at most 4 coordinate levels with every FP64 multiply and add
// rounded separately (namespaces l2 and l4: the reference's arithmetic), and
// for at most 2 levels with multiply-adds fused (l2f: FP32-table mode only,
// where results are compared statistically, not bit for bit); the functions
// in omc itself pick the build (transport_dispatch.cpp).
#define OMC_GPU_API(NS)                                                                     \
  namespace NS {                                                                            \
  struct GpuSim;                                                                            \
  GpuSim* gpu_create(const HModel& m, const GpuOptions& opt);                               \
  void gpu_destroy(GpuSim* g);                                                              \
  BatchStats gpu_run_batch(GpuSim* g, HModel& m, int batch, bool accumulate);               \
  BatchStats gpu_run_batch_profiled(GpuSim* g, HModel& m, int batch, bool accumulate);      \
  void gpu_fetch_tallies(GpuSim* g, HModel& m);                                             \
  void gpu_reset_tallies(GpuSim* g, HModel& m);                                             \
  void gpu_set_trace(GpuSim* g, long long n_hist, int cap, int batch, long long first);     \
  void gpu_get_trace(GpuSim* g, void* records, int* counts);                                \
  void gpu_set_ww_bounds(GpuSim* g, const double* lower, const double* upper, long long n); \
  void gpu_set_ww_on(GpuSim* g, bool on);                                                   \
  void gpu_update_magic(GpuSim* g, const MagicArgs& a, double* lower, double* upper);        \
  GenerationStats gpu_finish_generation(GpuSim* g, int batch);                               \
  void gpu_set_keff(GpuSim* g, double keff);                                                 \
  long long gpu_capacity(GpuSim* g);                                                        \
  void gpu_material_xs(GpuSim* g, long long n, const int* mat, const double* E, double* total, \
                       double* absorption, unsigned* grid_hash);                               \
  }

OMC_GPU_API(l2)
OMC_GPU_API(l4)
OMC_GPU_API(l2f)

GpuSim* gpu_create(const HModel& m, const GpuOptions& opt);
void gpu_destroy(GpuSim* g);
BatchStats gpu_run_batch(GpuSim* g, HModel& m, int batch, bool accumulate);
// Same batch launched kernel by kernel (no graph) with CUDA events around
// each kernel; identical results, slower, for per-kernel timing.
BatchStats gpu_run_batch_profiled(GpuSim* g, HModel& m, int batch, bool accumulate);
void gpu_fetch_tallies(GpuSim* g, HModel& m);
void gpu_reset_tallies(GpuSim* g, HModel& m);
void gpu_set_trace(GpuSim* g, long long n_hist, int cap, int batch, long long first);
void gpu_get_trace(GpuSim* g, void* records, int* counts);
void gpu_set_ww_bounds(GpuSim* g, const double* lower, const double* upper, long long n);
void gpu_set_ww_on(GpuSim* g, bool on);
// MAGIC update of the device's weight windows from the device's tally sums
// (no tally copy to the host); the new bounds are also copied into the host
// arrays lower / upper (e_bins x mesh_bins each).
void gpu_update_magic(GpuSim* g, const MagicArgs& a, double* lower, double* upper);
long long gpu_capacity(GpuSim* g);
// Eigenvalue run, after generation `batch`: reads its fission-bank size and
// k-effective sums, puts the bank in (parent, progeny) order, combs
// n_particles sites from it (src/eigenvalue.cpp:86-365, the tooth positions
// accumulated on the host as the reference accumulates them) and writes them
// as the next generation's source bank.
GenerationStats gpu_finish_generation(GpuSim* g, int batch);
// The k-effective the next generation's fission sites are sampled with.
void gpu_set_keff(GpuSim* g, double keff);
// Macroscopic total and absorption cross sections (and the nuclide grid-index
// hash) of the model's materials at (material index, E) pairs, evaluated on
// the device by the transport kernels' own lookup (host arrays of length n).
void gpu_material_xs(GpuSim* g, long long n, const int* mat, const double* E, double* total, double* absorption,
                     unsigned* grid_hash);
// coordinate depth of the kernels a simulation runs (2 or 4)
int gpu_levels(GpuSim* g);

}  // namespace omc
