/* C ABI of libopenmc_gb300.so — the GB300 event-based transport library.
 *
 * Every function below has the name, signature, argument meaning and return
 * convention of the reference C API it replaces (file:line in the reference
 * tree is given beside each); functions prefixed openmc_gb300_ are additions
 * with no reference counterpart.  Return value 0 means success; a negative
 * value is one of the exported OPENMC_E_* codes, with a message in
 * openmc_err_msg.
 */
#ifndef OPENMC_GB300_H
#define OPENMC_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes and message: include/openmc/capi.h:279-292, src/error.cpp:20-30 */
extern int OPENMC_E_UNASSIGNED;
extern int OPENMC_E_ALLOCATE;
extern int OPENMC_E_OUT_OF_BOUNDS;
extern int OPENMC_E_INVALID_SIZE;
extern int OPENMC_E_INVALID_ARGUMENT;
extern int OPENMC_E_INVALID_TYPE;
extern int OPENMC_E_INVALID_ID;
extern int OPENMC_E_GEOMETRY;
extern int OPENMC_E_DATA;
extern int OPENMC_E_PHYSICS;
extern int OPENMC_E_WARNING;
extern char openmc_err_msg[256];

/* ---- exported globals read through ctypes: include/openmc/settings.h:67-132,
 *      include/openmc/simulation.h:26-38, openmc/lib/__init__.py:40-50 */
extern bool event_based;
extern int64_t n_particles;
extern int32_t n_inactive;
extern int32_t gen_per_batch;
extern int32_t max_lost_particles;
extern double rel_max_lost_particles;
extern bool run_CE;
extern int verbosity;
extern bool weight_windows_on;
extern bool restart_run;
extern int current_batch;
extern int32_t n_realizations;  /* active batches realised (include/openmc/simulation.h) */
extern bool initialized;
extern int n_lost_particles;
extern int n_coord_levels;
extern bool DAGMC_ENABLED;
extern bool LIBMESH_ENABLED;
extern bool UWUW_ENABLED;

/* ---- lifecycle: include/openmc/capi.h:62-149, src/simulation.cpp:53-280 */
int openmc_init(int argc, char* argv[], const void* intracomm); /* capi.h:83 */
int openmc_run(void);                                           /* capi.h:142 */
int openmc_simulation_init(void);                               /* capi.h:149 */
int openmc_next_batch(int* status);                             /* capi.h:123 */
int openmc_simulation_finalize(void);                           /* capi.h:148 */
int openmc_finalize(void);                                      /* capi.h:62 */
int openmc_reset(void);                                         /* capi.h:140 */
int openmc_hard_reset(void);                                    /* capi.h:82 */
int openmc_reset_timers(void);                                  /* capi.h:141 */

/* ---- seeds: include/openmc/capi.h:77-78,144-145, src/random_lcg.cpp:126-144 */
int64_t openmc_get_seed(void);
void openmc_set_seed(int64_t new_seed);
uint64_t openmc_get_stride(void);
void openmc_set_stride(uint64_t new_stride);

/* ---- tallies: include/openmc/capi.h:79,81,168-174, src/tallies/tally.cpp:1554-1575.
 * openmc_tally_results returns a borrowed pointer to [bins][scores][3]
 * (VALUE, SUM, SUM_SQ) that stays valid until the next library call. */
int openmc_tally_results(int32_t index, double** ptr, size_t shape_[3]);
int openmc_get_tally_index(int32_t id, int32_t* index);
int openmc_tally_get_id(int32_t index, int32_t* id);
int openmc_tally_get_n_realizations(int32_t index, int32_t* n);
int openmc_global_tallies(double** ptr);
size_t tallies_size(void); /* src/tallies/tally.cpp:1584 */
int cells_size(void);           /* src/cell.cpp:1820 */
size_t n_materials(void);       /* src/material.cpp:1599 */
int n_meshes(void);             /* src/mesh.cpp:3900 */
size_t nuclides_size(void);     /* src/nuclide.cpp:1105 */
size_t tally_filters_size(void); /* src/tallies/filter.cpp:62 */

/* ---- weight windows: include/openmc/capi.h:184-221, src/weight_windows.cpp:1020-1340 */
size_t openmc_weight_windows_size(void);
int openmc_get_weight_windows_index(int32_t id, int32_t* idx);
int openmc_weight_windows_get_id(int32_t index, int32_t* id);
int openmc_weight_windows_get_bounds(int32_t index, const double** lower_bounds,
  const double** upper_bounds, size_t* size);
int openmc_weight_windows_set_bounds(int32_t index, const double* lower_bounds,
  const double* upper_bounds, size_t size);
int openmc_weight_windows_get_energy_bounds(int32_t index, const double** e_bounds,
  size_t* e_bounds_size);
int openmc_weight_windows_update_magic(int32_t ww_idx, int32_t tally_idx,
  const char* value, double threshold, double ratio);
int openmc_weight_windows_get_survival_ratio(int32_t index, double* ratio);
int openmc_weight_windows_get_max_split(int32_t index, int* max_split);
int openmc_weight_windows_get_mesh(int32_t index, int32_t* mesh_idx);

/* ---- GB300 additions (no reference counterpart) ----------------------- */
/* settings globals: FP32 tables (-1 = from <gb300_xs_precision>), particle
 * slots in HBM (0 = setting or automatic), XS-queue sort on/off */
extern int openmc_gb300_xs_fp32;
extern int64_t openmc_gb300_in_flight;
extern int openmc_gb300_sort;
/* bit 0: the cross-section event runs inside the advance kernel; bit 1 (with
 * bit 0): so does the surface crossing (default 3; 0: one kernel per event) */
extern int openmc_gb300_fuse;
extern int openmc_gb300_trace_batch;
extern int64_t openmc_gb300_trace_first;
/* 1: run the next batch kernel by kernel (no graph) with CUDA events around
 * each kernel; 2: run every batch that way (kernel profilers cannot look
 * inside graphs with conditional nodes); results are identical, per-kernel
 * times land in openmc_gb300_last_batch_detail */
extern int openmc_gb300_profile_next;
/* queue length at or below which, once every source particle has started,
 * the remaining histories run to completion one thread each (-1: default) */
extern int64_t openmc_gb300_tail_threshold;
/* entries of the device pool of banked secondaries (split particles); 0: automatic
 * (with weight windows max(64 x slots, 2^22), else 1024); 72 bytes per entry, 112 in
 * split-to-slots mode */
extern int64_t openmc_gb300_secondary_capacity;
/* 1: particles split by weight windows wait in a device ring and start in free
 * slots with their own tracking seeds (a hash of the parent's seed), so that a
 * split tree is tracked in parallel; 0 (default): the reference's behaviour,
 * each copy banked on the parent's LIFO stack and continued on the parent's
 * random stream after it (src/particle.cpp:417-473) */
extern int openmc_gb300_split_to_slots;
/* coordinate depth the transport kernels are built for: 0 (default) picks the
 * 2-level build for models nested at most 2 deep (per-level state in
 * registers) and the 4-level build otherwise; 4 forces the 4-level build */
extern int openmc_gb300_max_levels;
/* 1: each block of the event kernels copies the cell, surface, region-token,
 * universe and per-material nuclide tables into shared memory at entry (when
 * they fit in 32 KB) and reads them there; 0 (default): read through L1 from
 * global memory, where tables of a few KB stay resident */
extern int openmc_gb300_stage_tables;
/* 1 (default): FP32-table mode with at most 2 coordinate levels runs the
 * transport build whose FP64 multiply-adds are fused (one rounding each, the
 * default of most compilers); 0: the build that rounds every FP64 multiply
 * and add separately, as FP64-table mode always does */
extern int openmc_gb300_contract;
/* 1 (default): in the event loop, the advance kernel writes each flight as a
 * track record and a separate kernel scores the track-length tallies from
 * them (score_tracklength_tally, src/tallies/tally_scoring.cpp:2416-2541);
 * 0: the advance kernel scores them itself */
extern int openmc_gb300_defer_tally;

/* eigenvalue run: the track-length k of every generation so far (at most n
 * written; returns how many there are) and the last generation's
 * fission-bank size (src/eigenvalue.cpp:50-84 k_generation) */
int openmc_gb300_k_generation(double* k, int n, int64_t* fission_sites);
/* last batch: [ms, iterations, events, total_weight, leakage, lost, done, secondary-pool entries used,
 *  events of the longest history, its particle id] */
int openmc_gb300_last_batch(double* out);
/* [queue phase: xs events, xs recomputations, xs nuclide lookups, mesh
 *  segments, collision nuclide lookups, surface events, collisions; tail
 *  phase: the same seven; kernel ms: xs, advance, surface, collision, tail,
 *  refill, sort, other, track-length tally] (23 doubles) */
int openmc_gb300_last_batch_detail(double* out);
/* [time_active s, time_inactive s, wall_active s, particles/s (active), in-flight slots] */
int openmc_gb300_timing(double* out);
/* per-event traces for particle ids first..first+n_hist-1 of the traced batch,
 * cap records each (48-byte records) */
int openmc_gb300_set_trace(int64_t n_hist, int cap);
int openmc_gb300_get_trace(void* records, int32_t* counts);
int openmc_gb300_set_weight_windows_on(int on);
/* [n_nuclides, n_materials, n_cells, n_surfaces, n_tallies, log_grid_bins, batches, coord_levels] */
int openmc_gb300_model_info(int64_t* out);
/* macroscopic total and absorption cross sections of the initialised
 * simulation's materials (0-based material indices) at energies E [eV],
 * evaluated on the device by the transport kernels' own lookup and tables
 * (FP32 or FP64 as openmc_gb300_xs_fp32 chose), with the hash of the
 * nuclides' grid indices; Material::calculate_neutron_xs
 * (src/material.cpp:829-901) per pair.  Host arrays of length n. */
int openmc_gb300_material_xs(int64_t n, const int32_t* material, const double* E, double* total,
                             double* absorption, uint32_t* grid_hash);

/* macroscopic-XS lookup on flat 5-channel tables; counterpart of
 * Material::calculate_neutron_xs (src/material.cpp:829-901) per lookup.
 * Material indices outside [0, n_mat): openmc_gb300_xs_lookup (host
 * buffers) returns OPENMC_E_OUT_OF_BOUNDS before any work; the device-buffer
 * entry points cannot check before queuing the work, so such a lookup reads
 * no table and gets NaN results and grid hash 0. */
int openmc_gb300_xs_tables_create(int n_nuc, int G, const double* energy, const double* xs,
  int n_mat, const int32_t* mat_off, const int32_t* mat_nuc, const double* mat_dens,
  int n_log_bins, int fp32, int64_t max_lookups, void** handle);
int openmc_gb300_xs_tables_free(void* handle);
int openmc_gb300_xs_lookup(void* handle, int64_t n, const int32_t* mat, const double* E,
  double* out, int32_t* grid_hash, int sort);
int openmc_gb300_xs_lookup_device(void* handle, int64_t n, const int32_t* d_mat,
  const double* d_E, double* d_out, int32_t* d_grid_hash, int sort);
int openmc_gb300_xs_last_times(void* handle, float* ms);
int openmc_gb300_xs_stream(void* handle, void** stream);
/* No counterpart in the reference: the sorted lookups of
 * openmc_gb300_xs_lookup_device for callers that cannot allocate device
 * memory during the call (a memory budget or a pool they do not own).  It
 * allocates nothing; its sort scratch is a static device array of the
 * library (about 16 MiB held by every GPU that loads it).  At most 4,194,304
 * lookups per call and 64 materials, else OPENMC_E_INVALID_ARGUMENT.  The
 * first call on a device looks up the array's address and should come before
 * any stream capture; calls that overlap on the GPU share the array and race.
 * Work is queued on `stream` (cudaStream_t, NULL = default) without waiting. */
int openmc_gb300_xs_lookup_noalloc(void* handle, int64_t n, const int32_t* d_mat,
  const double* d_E, double* d_out, int32_t* d_grid_hash, void* stream);

/* Learned weight windows (no reference counterpart; its output replaces the
 * MAGIC bounds of WeightWindows::update_weights, src/weight_windows.cpp:502-755,
 * and is consumed unchanged by apply_weight_windows, :56-146).
 * Importance network (x, y, z, log E) -> log flux: 4 -> 128 -> 128 -> 128 -> 1,
 * SiLU, BF16 tcgen05 products accumulating in FP32, FP32 master weights,
 * full-batch Adam (beta 0.9 / 0.999, eps 1e-8).  Parameters are one flat FP32
 * vector: W1[128][4], b1[128], W2[128][128], b2, W3[128][128], b3, w4[128], b4.
 * Host pointers throughout; x4 is n rows of 4 features. */
int openmc_gb300_mlp_n_params(void);
int openmc_gb300_mlp_create(int64_t max_rows, uint64_t seed, void** handle);
int openmc_gb300_mlp_free(void* handle);
int openmc_gb300_mlp_set_data(void* handle, int64_t n, const float* x4, const float* target,
  const float* weight);
int openmc_gb300_mlp_train(void* handle, int steps, double lr, float* loss_history);
int openmc_gb300_mlp_gradients(void* handle, float* grad, float* loss);
int openmc_gb300_mlp_predict(void* handle, int64_t n, const float* x4, float* y);
int openmc_gb300_mlp_get_params(void* handle, float* params, int64_t n);
int openmc_gb300_mlp_set_params(void* handle, const float* params, int64_t n);
int openmc_gb300_mlp_last_ms(void* handle, float* ms);
/* 1 (default): every training step and query is one fused kernel per
 * 128-row tile (activations of all layers kept in shared and tensor memory);
 * 0: one kernel per layer product, activations through device memory. */
extern int openmc_gb300_mlp_fused;

/* ---- model queries the reference's Python bindings use (openmc/lib/cell.py,
 *      material.py, mesh.py, filter.py, tally.py, nuclide.py, core.py),
 *      answered from the loaded model; prototypes of include/openmc/capi.h */
bool openmc_master(void);                                              /* src/initialize.cpp */
bool openmc_is_statepoint_batch(void);                                 /* src/state_point.cpp */
int openmc_get_n_batches(int* n_batches, bool get_max_batches);        /* src/settings.cpp:1319-1324 */
int openmc_set_n_batches(int32_t n_batches, bool set_max_batches, bool add_statepoint_batch);  /* :1285-1317 */
int openmc_get_keff(double k_combined[]);                              /* src/eigenvalue.cpp:420-579 */
/* statepoint file format 18.1 (tallies, k-effective, global tallies; no source
 * bank); filename NULL: statepoint.<batch>.h5 in the output path */
int openmc_statepoint_write(const char* filename, bool* write_source);  /* src/state_point.cpp:36-357 */
int openmc_get_cell_index(int32_t id, int32_t* index);                 /* src/cell.cpp */
int openmc_cell_get_id(int32_t index, int32_t* id);
int openmc_cell_get_translation(int32_t index, double xyz[]);
int openmc_cell_get_name(int32_t index, const char** name);
int openmc_get_material_index(int32_t id, int32_t* index);             /* src/material.cpp */
int openmc_material_get_id(int32_t index, int32_t* id);
int openmc_material_get_name(int32_t index, const char** name);
int openmc_material_get_densities(int32_t index, const int** nuclides, const double** densities, int* n);  /* :1389-1407 */
int openmc_material_get_density(int32_t index, double* density);      /* :1409-1419 */
int openmc_cell_get_fill(int32_t index, int* type, int32_t** indices, int32_t* n);  /* src/cell.cpp */
int openmc_cell_get_num_instances(int32_t index, int32_t* num_instances);  /* src/cell.cpp */
int openmc_cell_bounding_box(const int32_t index, double* llc, double* urc);  /* src/cell.cpp */
int openmc_global_bounding_box(double* llc, double* urc);              /* src/geometry.cpp */
int openmc_get_nuclide_index(const char name[], int* index);           /* src/nuclide.cpp */
int openmc_nuclide_name(int index, const char** name);
int openmc_get_mesh_index(int32_t id, int32_t* index);                 /* src/mesh.cpp */
int openmc_mesh_get_id(int32_t index, int32_t* id);
int openmc_mesh_get_type(int32_t index, char* type);                   /* :2285-2293 */
int openmc_mesh_get_n_elements(int32_t index, size_t* n);
int openmc_mesh_bounding_box(int32_t index, double* ll, double* ur);
int openmc_regular_mesh_get_dimension(int32_t index, int** dims, int* n);  /* :2508-2517 */
int openmc_regular_mesh_get_params(int32_t index, double** ll, double** ur, double** width, int* n);  /* :2534-2555 */
int openmc_get_filter_index(int32_t id, int32_t* index);               /* src/tallies/filter.cpp */
int openmc_filter_get_id(int32_t index, int32_t* id);
int openmc_filter_get_type(int32_t index, char* type);                 /* :234-241 */
int openmc_filter_get_num_bins(int32_t index, int* n_bins);            /* :243-250 */
int openmc_energy_filter_get_bins(int32_t index, const double** energies, size_t* n);  /* filter_energy.cpp */
int openmc_mesh_filter_get_mesh(int32_t index, int32_t* index_mesh);   /* filter_mesh.cpp */
int openmc_cell_filter_get_bins(int32_t index, const int32_t** cells, int32_t* n);  /* filter_cell.cpp */
int openmc_material_filter_get_bins(int32_t index, const int32_t** bins, size_t* n);  /* filter_material.cpp */
int openmc_mesh_filter_get_translation(int32_t index, double translation[3]);  /* filter_mesh.cpp */
int openmc_particle_filter_get_bins(int32_t idx, int bins[]);          /* filter_particle.cpp */
int openmc_tally_get_type(int32_t index, int32_t* type);               /* src/tallies/tally.cpp */
int openmc_tally_get_estimator(int32_t index, int* estimator);
int openmc_tally_get_active(int32_t index, bool* active);
int openmc_tally_get_writable(int32_t index, bool* writable);
int openmc_tally_get_multiply_density(int32_t index, bool* value);
int openmc_tally_get_filters(int32_t index, const int32_t** indices, size_t* n);
int openmc_tally_get_scores(int32_t index, int** scores, int* n);
int openmc_tally_get_nuclides(int32_t index, int** nuclides, int* n);

/* ---- every other entry point the reference's Python bindings name:
 *      include/openmc_gb300_offpath.h (each returns OPENMC_E_UNASSIGNED) */

#ifdef __cplusplus
}
#endif

#endif /* OPENMC_GB300_H */
