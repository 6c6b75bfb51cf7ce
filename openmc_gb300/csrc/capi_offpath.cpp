// Generated by make_capi_offpath.py: openmc.lib entry points outside the
// event-based fixed-source transport path (model mutation, plotting,
// volumes, depletion, CMFD, DAGMC, statepoints, source banks, other mesh and
// filter types).  The reference binds every one of them at import
// (openmc/lib/*.py); here each reports that it is not available.
#include <cstddef>
#include <cstdint>
#include <cstdio>

extern "C" {
extern int OPENMC_E_UNASSIGNED;
extern char openmc_err_msg[256];
}

namespace {
struct Position {
  double x, y, z;
};

int off_path(const char* name)
{
  std::snprintf(openmc_err_msg, 256, "%s is not available in the GB300 transport library "
                "(outside the event-based fixed-source path).", name);
  return OPENMC_E_UNASSIGNED;
}
}  // namespace

extern "C" {

void calc_zn(int n, double rho, double phi, double zn[])
{
  off_path("calc_zn");
}

void calc_zn_rad(int n, double rho, double zn_rad[])
{
  off_path("calc_zn_rad");
}

int openmc_calculate_volumes()
{ return off_path("openmc_calculate_volumes"); }

int openmc_cell_get_density(int32_t index, const int32_t* instance, double* rho)
{ return off_path("openmc_cell_get_density"); }

int openmc_cell_get_rotation(int32_t index, double rot[], size_t* n)
{ return off_path("openmc_cell_get_rotation"); }

int openmc_cell_get_temperature(int32_t index, const int32_t* instance, double* T)
{ return off_path("openmc_cell_get_temperature"); }

int openmc_cell_set_density(int32_t index, double rho, const int32_t* instance, bool set_contained)
{ return off_path("openmc_cell_set_density"); }

int openmc_cell_set_fill(int32_t index, int type, int32_t n, const int32_t* indices)
{ return off_path("openmc_cell_set_fill"); }

int openmc_cell_set_id(int32_t index, int32_t id)
{ return off_path("openmc_cell_set_id"); }

int openmc_cell_set_name(int32_t index, const char* name)
{ return off_path("openmc_cell_set_name"); }

int openmc_cell_set_rotation(int32_t index, const double rot[], size_t rot_len)
{ return off_path("openmc_cell_set_rotation"); }

int openmc_cell_set_temperature(int32_t index, double T, const int32_t* instance, bool set_contained)
{ return off_path("openmc_cell_set_temperature"); }

int openmc_cell_set_translation(int32_t index, const double xyz[])
{ return off_path("openmc_cell_set_translation"); }

void openmc_cmfd_reweight(const bool feedback, const double* cmfd_src)
{
  off_path("openmc_cmfd_reweight");
}

int openmc_cylindrical_mesh_get_grid(int32_t index, double** grid_x, int* nx, double** grid_y, int* ny, double** grid_z, int* nz)
{ return off_path("openmc_cylindrical_mesh_get_grid"); }

int openmc_cylindrical_mesh_set_grid(int32_t index, const double* grid_x, const int nx, const double* grid_y, const int ny, const double* grid_z, const int nz)
{ return off_path("openmc_cylindrical_mesh_set_grid"); }

int openmc_dagmc_universe_get_cell_ids(int32_t univ_id, int32_t* ids, size_t* n)
{ return off_path("openmc_dagmc_universe_get_cell_ids"); }

int openmc_dagmc_universe_get_num_cells(int32_t univ_id, size_t* n)
{ return off_path("openmc_dagmc_universe_get_num_cells"); }

int openmc_energy_filter_set_bins(int32_t index, size_t n, const double* energies)
{ return off_path("openmc_energy_filter_set_bins"); }

int openmc_energyfunc_filter_get_energy(int32_t index, size_t* n, const double** energy)
{ return off_path("openmc_energyfunc_filter_get_energy"); }

int openmc_energyfunc_filter_get_interpolation(int32_t index, int* interp)
{ return off_path("openmc_energyfunc_filter_get_interpolation"); }

int openmc_energyfunc_filter_get_y(int32_t index, size_t* n, const double** y)
{ return off_path("openmc_energyfunc_filter_get_y"); }

int openmc_energyfunc_filter_set_data(int32_t index, size_t n, const double* energies, const double* y)
{ return off_path("openmc_energyfunc_filter_set_data"); }

int openmc_energyfunc_filter_set_interpolation(int32_t index, const char* interp)
{ return off_path("openmc_energyfunc_filter_set_interpolation"); }

int openmc_extend_cells(int32_t n, int32_t* index_start, int32_t* index_end)
{ return off_path("openmc_extend_cells"); }

int openmc_extend_materials(int32_t n, int32_t* index_start, int32_t* index_end)
{ return off_path("openmc_extend_materials"); }

int openmc_extend_meshes(int32_t n, const char* type, int32_t* index_start, int32_t* index_end)
{ return off_path("openmc_extend_meshes"); }

int openmc_extend_tallies(int32_t n, int32_t* index_start, int32_t* index_end)
{ return off_path("openmc_extend_tallies"); }

int openmc_extend_weight_windows(int32_t n, int32_t* index_start, int32_t* index_end)
{ return off_path("openmc_extend_weight_windows"); }

int openmc_filter_set_id(int32_t index, int32_t id)
{ return off_path("openmc_filter_set_id"); }

int openmc_find_cell(const double* xyz, int32_t* index, int32_t* instance)
{ return off_path("openmc_find_cell"); }

int openmc_id_map(const void* slice, int32_t* data_out)
{ return off_path("openmc_id_map"); }

void openmc_initialize_linsolver(const int* indptr, int len_indptr, const int* indices, int n_elements, int dim, double spectral, const int* map, bool use_all_threads)
{
  off_path("openmc_initialize_linsolver");
}

void openmc_initialize_mesh_egrid(const int meshtally_id, const int* cmfd_indices, const double norm)
{
  off_path("openmc_initialize_mesh_egrid");
}

int openmc_legendre_filter_get_order(int32_t index, int* order)
{ return off_path("openmc_legendre_filter_get_order"); }

int openmc_legendre_filter_set_order(int32_t index, int order)
{ return off_path("openmc_legendre_filter_set_order"); }

int openmc_load_nuclide(const char* name, const double* temps, int n)
{ return off_path("openmc_load_nuclide"); }

int openmc_material_add_nuclide(int32_t index, const char name[], double density)
{ return off_path("openmc_material_add_nuclide"); }

int openmc_material_filter_set_bins(int32_t index, size_t n, const int32_t* bins)
{ return off_path("openmc_material_filter_set_bins"); }

int openmc_material_get_depletable(int32_t index, bool* depletable)
{ return off_path("openmc_material_get_depletable"); }

int openmc_material_get_temperature(int32_t index, double* temperature)
{ return off_path("openmc_material_get_temperature"); }

int openmc_material_get_volume(int32_t index, double* volume)
{ return off_path("openmc_material_get_volume"); }

int openmc_material_set_densities(int32_t index, int n, const char** name, const double* density)
{ return off_path("openmc_material_set_densities"); }

int openmc_material_set_density(int32_t index, double density, const char* units)
{ return off_path("openmc_material_set_density"); }

int openmc_material_set_depletable(int32_t index, bool depletable)
{ return off_path("openmc_material_set_depletable"); }

int openmc_material_set_id(int32_t index, int32_t id)
{ return off_path("openmc_material_set_id"); }

int openmc_material_set_name(int32_t index, const char* name)
{ return off_path("openmc_material_set_name"); }

int openmc_material_set_volume(int32_t index, double volume)
{ return off_path("openmc_material_set_volume"); }

int openmc_mesh_filter_get_rotation(int32_t index, double rot[], size_t* n)
{ return off_path("openmc_mesh_filter_get_rotation"); }

int openmc_mesh_filter_set_mesh(int32_t index, int32_t index_mesh)
{ return off_path("openmc_mesh_filter_set_mesh"); }

int openmc_mesh_filter_set_rotation(int32_t index, const double rot[], size_t rot_len)
{ return off_path("openmc_mesh_filter_set_rotation"); }

int openmc_mesh_filter_set_translation(int32_t index, double translation[3])
{ return off_path("openmc_mesh_filter_set_translation"); }

int openmc_mesh_get_plot_bins(int32_t index, Position origin, Position width, int basis, int* pixels, int32_t* data)
{ return off_path("openmc_mesh_get_plot_bins"); }

int openmc_mesh_get_volumes(int32_t index, double* volumes)
{ return off_path("openmc_mesh_get_volumes"); }

int openmc_mesh_material_volumes(int32_t index, int nx, int ny, int nz, int max_mats, int32_t* materials, double* volumes)
{ return off_path("openmc_mesh_material_volumes"); }

int openmc_mesh_set_id(int32_t index, int32_t id)
{ return off_path("openmc_mesh_set_id"); }

int openmc_meshborn_filter_get_mesh(int32_t index, int32_t* index_mesh)
{ return off_path("openmc_meshborn_filter_get_mesh"); }

int openmc_meshborn_filter_get_translation(int32_t index, double translation[3])
{ return off_path("openmc_meshborn_filter_get_translation"); }

int openmc_meshborn_filter_set_mesh(int32_t index, int32_t index_mesh)
{ return off_path("openmc_meshborn_filter_set_mesh"); }

int openmc_meshborn_filter_set_translation(int32_t index, double translation[3])
{ return off_path("openmc_meshborn_filter_set_translation"); }

int openmc_meshsurface_filter_get_mesh(int32_t index, int32_t* index_mesh)
{ return off_path("openmc_meshsurface_filter_get_mesh"); }

int openmc_meshsurface_filter_get_translation(int32_t index, double translation[3])
{ return off_path("openmc_meshsurface_filter_get_translation"); }

int openmc_meshsurface_filter_set_mesh(int32_t index, int32_t index_mesh)
{ return off_path("openmc_meshsurface_filter_set_mesh"); }

int openmc_meshsurface_filter_set_translation(int32_t index, double translation[3])
{ return off_path("openmc_meshsurface_filter_set_translation"); }

int openmc_new_filter(const char* type, int32_t* index)
{ return off_path("openmc_new_filter"); }

int openmc_nuclide_collapse_rate(int index, int MT, double temperature, const double* energy, const double* flux, int n, double* xs)
{ return off_path("openmc_nuclide_collapse_rate"); }

int openmc_plot_geometry()
{ return off_path("openmc_plot_geometry"); }

int openmc_properties_export(const char* filename)
{ return off_path("openmc_properties_export"); }

int openmc_properties_import(const char* filename)
{ return off_path("openmc_properties_import"); }

int openmc_property_map(const void* slice, double* data_out)
{ return off_path("openmc_property_map"); }

int openmc_rectilinear_mesh_get_grid(int32_t index, double** grid_x, int* nx, double** grid_y, int* ny, double** grid_z, int* nz)
{ return off_path("openmc_rectilinear_mesh_get_grid"); }

int openmc_rectilinear_mesh_set_grid(int32_t index, const double* grid_x, const int nx, const double* grid_y, const int ny, const double* grid_z, const int nz)
{ return off_path("openmc_rectilinear_mesh_set_grid"); }

int openmc_regular_mesh_set_dimension(int32_t index, int n, const int* dims)
{ return off_path("openmc_regular_mesh_set_dimension"); }

int openmc_regular_mesh_set_params(int32_t index, int n, const double* ll, const double* ur, const double* width)
{ return off_path("openmc_regular_mesh_set_params"); }

int openmc_remove_tally(int32_t index)
{ return off_path("openmc_remove_tally"); }

int openmc_run_linsolver(const double* A_data, const double* b, double* x, double tol)
{ return off_path("openmc_run_linsolver"); }

int openmc_sample_external_source(size_t n, uint64_t* seed, void* sites)
{ return off_path("openmc_sample_external_source"); }

int openmc_source_bank(void** ptr, int64_t* n)
{ return off_path("openmc_source_bank"); }

int openmc_spatial_legendre_filter_get_order(int32_t index, int* order)
{ return off_path("openmc_spatial_legendre_filter_get_order"); }

int openmc_spatial_legendre_filter_set_order(int32_t index, int order)
{ return off_path("openmc_spatial_legendre_filter_set_order"); }

int openmc_spherical_mesh_get_grid(int32_t index, double** grid_x, int* nx, double** grid_y, int* ny, double** grid_z, int* nz)
{ return off_path("openmc_spherical_mesh_get_grid"); }

int openmc_spherical_mesh_set_grid(int32_t index, const double* grid_x, const int nx, const double* grid_y, const int ny, const double* grid_z, const int nz)
{ return off_path("openmc_spherical_mesh_set_grid"); }

int openmc_sphharm_filter_get_order(int32_t index, int* order)
{ return off_path("openmc_sphharm_filter_get_order"); }

int openmc_sphharm_filter_set_order(int32_t index, int order)
{ return off_path("openmc_sphharm_filter_set_order"); }

int openmc_statepoint_load(const char* filename)
{ return off_path("openmc_statepoint_load"); }

int openmc_tally_reset(int32_t index)
{ return off_path("openmc_tally_reset"); }

int openmc_tally_set_active(int32_t index, bool active)
{ return off_path("openmc_tally_set_active"); }

int openmc_tally_set_estimator(int32_t index, const char* estimator)
{ return off_path("openmc_tally_set_estimator"); }

int openmc_tally_set_filters(int32_t index, size_t n, const int32_t* indices)
{ return off_path("openmc_tally_set_filters"); }

int openmc_tally_set_id(int32_t index, int32_t id)
{ return off_path("openmc_tally_set_id"); }

int openmc_tally_set_multiply_density(int32_t index, bool value)
{ return off_path("openmc_tally_set_multiply_density"); }

int openmc_tally_set_nuclides(int32_t index, int n, const char** nuclides)
{ return off_path("openmc_tally_set_nuclides"); }

int openmc_tally_set_scores(int32_t index, int n, const char** scores)
{ return off_path("openmc_tally_set_scores"); }

int openmc_tally_set_type(int32_t index, const char* type)
{ return off_path("openmc_tally_set_type"); }

int openmc_tally_set_writable(int32_t index, bool writable)
{ return off_path("openmc_tally_set_writable"); }

int openmc_weight_windows_export(const char* filename)
{ return off_path("openmc_weight_windows_export"); }

int openmc_weight_windows_get_max_lower_bound_ratio(int32_t index, double* lb_ratio)
{ return off_path("openmc_weight_windows_get_max_lower_bound_ratio"); }

int openmc_weight_windows_get_particle(int32_t index, int* particle)
{ return off_path("openmc_weight_windows_get_particle"); }

int openmc_weight_windows_get_weight_cutoff(int32_t index, double* cutoff)
{ return off_path("openmc_weight_windows_get_weight_cutoff"); }

int openmc_weight_windows_import(const char* filename)
{ return off_path("openmc_weight_windows_import"); }

int openmc_weight_windows_set_energy_bounds(int32_t index, double* e_bounds, size_t e_bounds_size)
{ return off_path("openmc_weight_windows_set_energy_bounds"); }

int openmc_weight_windows_set_id(int32_t index, int32_t id)
{ return off_path("openmc_weight_windows_set_id"); }

int openmc_weight_windows_set_max_lower_bound_ratio(int32_t index, double lb_ratio)
{ return off_path("openmc_weight_windows_set_max_lower_bound_ratio"); }

int openmc_weight_windows_set_max_split(int32_t index, int max_split)
{ return off_path("openmc_weight_windows_set_max_split"); }

int openmc_weight_windows_set_mesh(int32_t index, int32_t mesh_idx)
{ return off_path("openmc_weight_windows_set_mesh"); }

int openmc_weight_windows_set_particle(int32_t index, int particle)
{ return off_path("openmc_weight_windows_set_particle"); }

int openmc_weight_windows_set_survival_ratio(int32_t index, double ratio)
{ return off_path("openmc_weight_windows_set_survival_ratio"); }

int openmc_weight_windows_set_weight_cutoff(int32_t index, double cutoff)
{ return off_path("openmc_weight_windows_set_weight_cutoff"); }

int openmc_zernike_filter_get_order(int32_t index, int* order)
{ return off_path("openmc_zernike_filter_get_order"); }

int openmc_zernike_filter_set_order(int32_t index, int order)
{ return off_path("openmc_zernike_filter_set_order"); }

}  // extern "C"
