/* Generated by openmc_gb300/csrc/make_capi_offpath.py: the openmc.lib entry
 * points outside the event-based fixed-source path that this library
 * exports only so that the reference's Python bindings (openmc/lib/*.py)
 * load it.  Prototypes as in the reference's include/openmc/capi.h (or its
 * src/ definitions); every call returns OPENMC_E_UNASSIGNED with a message
 * in openmc_err_msg (void functions only set the message, bool functions
 * return false). */
#ifndef OPENMC_GB300_OFFPATH_H
#define OPENMC_GB300_OFFPATH_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double x, y, z; } openmc_gb300_position;  /* Position */

void calc_zn(int n, double rho, double phi, double zn[]);
void calc_zn_rad(int n, double rho, double zn_rad[]);
int openmc_calculate_volumes(void);
int openmc_cell_get_density(int32_t index, const int32_t* instance, double* rho);
int openmc_cell_get_rotation(int32_t index, double rot[], size_t* n);
int openmc_cell_get_temperature(int32_t index, const int32_t* instance, double* T);
int openmc_cell_set_density(int32_t index, double rho, const int32_t* instance, bool set_contained);
int openmc_cell_set_fill(int32_t index, int type, int32_t n, const int32_t* indices);
int openmc_cell_set_id(int32_t index, int32_t id);
int openmc_cell_set_name(int32_t index, const char* name);
int openmc_cell_set_rotation(int32_t index, const double rot[], size_t rot_len);
int openmc_cell_set_temperature(int32_t index, double T, const int32_t* instance, bool set_contained);
int openmc_cell_set_translation(int32_t index, const double xyz[]);
void openmc_cmfd_reweight(const bool feedback, const double* cmfd_src);
int openmc_cylindrical_mesh_get_grid(int32_t index, double** grid_x, int* nx, double** grid_y, int* ny, double** grid_z, int* nz);
int openmc_cylindrical_mesh_set_grid(int32_t index, const double* grid_x, const int nx, const double* grid_y, const int ny, const double* grid_z, const int nz);
int openmc_dagmc_universe_get_cell_ids(int32_t univ_id, int32_t* ids, size_t* n);
int openmc_dagmc_universe_get_num_cells(int32_t univ_id, size_t* n);
int openmc_energy_filter_set_bins(int32_t index, size_t n, const double* energies);
int openmc_energyfunc_filter_get_energy(int32_t index, size_t* n, const double** energy);
int openmc_energyfunc_filter_get_interpolation(int32_t index, int* interp);
int openmc_energyfunc_filter_get_y(int32_t index, size_t* n, const double** y);
int openmc_energyfunc_filter_set_data(int32_t index, size_t n, const double* energies, const double* y);
int openmc_energyfunc_filter_set_interpolation(int32_t index, const char* interp);
int openmc_extend_cells(int32_t n, int32_t* index_start, int32_t* index_end);
int openmc_extend_materials(int32_t n, int32_t* index_start, int32_t* index_end);
int openmc_extend_meshes(int32_t n, const char* type, int32_t* index_start, int32_t* index_end);
int openmc_extend_tallies(int32_t n, int32_t* index_start, int32_t* index_end);
int openmc_extend_weight_windows(int32_t n, int32_t* index_start, int32_t* index_end);
int openmc_filter_set_id(int32_t index, int32_t id);
int openmc_find_cell(const double* xyz, int32_t* index, int32_t* instance);
int openmc_id_map(const void* slice, int32_t* data_out);
void openmc_initialize_linsolver(const int* indptr, int len_indptr, const int* indices, int n_elements, int dim, double spectral, const int* map, bool use_all_threads);
void openmc_initialize_mesh_egrid(const int meshtally_id, const int* cmfd_indices, const double norm);
int openmc_legendre_filter_get_order(int32_t index, int* order);
int openmc_legendre_filter_set_order(int32_t index, int order);
int openmc_load_nuclide(const char* name, const double* temps, int n);
int openmc_material_add_nuclide(int32_t index, const char name[], double density);
int openmc_material_filter_set_bins(int32_t index, size_t n, const int32_t* bins);
int openmc_material_get_depletable(int32_t index, bool* depletable);
int openmc_material_get_temperature(int32_t index, double* temperature);
int openmc_material_get_volume(int32_t index, double* volume);
int openmc_material_set_densities(int32_t index, int n, const char** name, const double* density);
int openmc_material_set_density(int32_t index, double density, const char* units);
int openmc_material_set_depletable(int32_t index, bool depletable);
int openmc_material_set_id(int32_t index, int32_t id);
int openmc_material_set_name(int32_t index, const char* name);
int openmc_material_set_volume(int32_t index, double volume);
int openmc_mesh_filter_get_rotation(int32_t index, double rot[], size_t* n);
int openmc_mesh_filter_set_mesh(int32_t index, int32_t index_mesh);
int openmc_mesh_filter_set_rotation(int32_t index, const double rot[], size_t rot_len);
int openmc_mesh_filter_set_translation(int32_t index, double translation[3]);
int openmc_mesh_get_plot_bins(int32_t index, openmc_gb300_position origin, openmc_gb300_position width, int basis, int* pixels, int32_t* data);
int openmc_mesh_get_volumes(int32_t index, double* volumes);
int openmc_mesh_material_volumes(int32_t index, int nx, int ny, int nz, int max_mats, int32_t* materials, double* volumes);
int openmc_mesh_set_id(int32_t index, int32_t id);
int openmc_meshborn_filter_get_mesh(int32_t index, int32_t* index_mesh);
int openmc_meshborn_filter_get_translation(int32_t index, double translation[3]);
int openmc_meshborn_filter_set_mesh(int32_t index, int32_t index_mesh);
int openmc_meshborn_filter_set_translation(int32_t index, double translation[3]);
int openmc_meshsurface_filter_get_mesh(int32_t index, int32_t* index_mesh);
int openmc_meshsurface_filter_get_translation(int32_t index, double translation[3]);
int openmc_meshsurface_filter_set_mesh(int32_t index, int32_t index_mesh);
int openmc_meshsurface_filter_set_translation(int32_t index, double translation[3]);
int openmc_new_filter(const char* type, int32_t* index);
int openmc_nuclide_collapse_rate(int index, int MT, double temperature, const double* energy, const double* flux, int n, double* xs);
int openmc_plot_geometry(void);
int openmc_properties_export(const char* filename);
int openmc_properties_import(const char* filename);
int openmc_property_map(const void* slice, double* data_out);
int openmc_rectilinear_mesh_get_grid(int32_t index, double** grid_x, int* nx, double** grid_y, int* ny, double** grid_z, int* nz);
int openmc_rectilinear_mesh_set_grid(int32_t index, const double* grid_x, const int nx, const double* grid_y, const int ny, const double* grid_z, const int nz);
int openmc_regular_mesh_set_dimension(int32_t index, int n, const int* dims);
int openmc_regular_mesh_set_params(int32_t index, int n, const double* ll, const double* ur, const double* width);
int openmc_remove_tally(int32_t index);
int openmc_run_linsolver(const double* A_data, const double* b, double* x, double tol);
int openmc_sample_external_source(size_t n, uint64_t* seed, void* sites);
int openmc_source_bank(void** ptr, int64_t* n);
int openmc_spatial_legendre_filter_get_order(int32_t index, int* order);
int openmc_spatial_legendre_filter_set_order(int32_t index, int order);
int openmc_spherical_mesh_get_grid(int32_t index, double** grid_x, int* nx, double** grid_y, int* ny, double** grid_z, int* nz);
int openmc_spherical_mesh_set_grid(int32_t index, const double* grid_x, const int nx, const double* grid_y, const int ny, const double* grid_z, const int nz);
int openmc_sphharm_filter_get_order(int32_t index, int* order);
int openmc_sphharm_filter_set_order(int32_t index, int order);
int openmc_statepoint_load(const char* filename);
int openmc_tally_reset(int32_t index);
int openmc_tally_set_active(int32_t index, bool active);
int openmc_tally_set_estimator(int32_t index, const char* estimator);
int openmc_tally_set_filters(int32_t index, size_t n, const int32_t* indices);
int openmc_tally_set_id(int32_t index, int32_t id);
int openmc_tally_set_multiply_density(int32_t index, bool value);
int openmc_tally_set_nuclides(int32_t index, int n, const char** nuclides);
int openmc_tally_set_scores(int32_t index, int n, const char** scores);
int openmc_tally_set_type(int32_t index, const char* type);
int openmc_tally_set_writable(int32_t index, bool writable);
int openmc_weight_windows_export(const char* filename);
int openmc_weight_windows_get_max_lower_bound_ratio(int32_t index, double* lb_ratio);
int openmc_weight_windows_get_particle(int32_t index, int* particle);
int openmc_weight_windows_get_weight_cutoff(int32_t index, double* cutoff);
int openmc_weight_windows_import(const char* filename);
int openmc_weight_windows_set_energy_bounds(int32_t index, double* e_bounds, size_t e_bounds_size);
int openmc_weight_windows_set_id(int32_t index, int32_t id);
int openmc_weight_windows_set_max_lower_bound_ratio(int32_t index, double lb_ratio);
int openmc_weight_windows_set_max_split(int32_t index, int max_split);
int openmc_weight_windows_set_mesh(int32_t index, int32_t mesh_idx);
int openmc_weight_windows_set_particle(int32_t index, int particle);
int openmc_weight_windows_set_survival_ratio(int32_t index, double ratio);
int openmc_weight_windows_set_weight_cutoff(int32_t index, double cutoff);
int openmc_zernike_filter_get_order(int32_t index, int* order);
int openmc_zernike_filter_set_order(int32_t index, int order);

#ifdef __cplusplus
}
#endif
#endif
