// Model queries of the openmc.lib C API that the reference's Python bindings
// bind at import (openmc/lib/cell.py, material.py, mesh.py, filter.py,
// tally.py, nuclide.py, core.py): index and ID lookups, regular-mesh
// parameters, filter and tally descriptions, batch counts and k-effective,
// answered from the loaded host model.  Names, arguments, borrowed-pointer
// returns and error codes follow include/openmc/capi.h and the reference
// functions cited beside each group.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "host_model.h"

namespace omc {
HModel* capi_model();
int capi_fail(int code, const std::string& msg);
}  // namespace omc

extern "C" {
extern int OPENMC_E_ALLOCATE;
extern int OPENMC_E_OUT_OF_BOUNDS;
extern int OPENMC_E_INVALID_ARGUMENT;
extern int OPENMC_E_INVALID_TYPE;
extern int OPENMC_E_INVALID_ID;
extern int OPENMC_E_DATA;
extern int32_t n_inactive;
extern int32_t n_realizations;
extern double keff;
extern double keff_std;
extern int current_batch;
}

namespace {

using omc::capi_fail;
using omc::HModel;

// The loaded model, or an OPENMC_E_ALLOCATE error as the reference returns
// before openmc_init.
HModel* model_or_fail(int& rc)
{
  HModel* m = omc::capi_model();
  rc = m ? 0 : capi_fail(OPENMC_E_ALLOCATE, "OpenMC has not been initialized.");
  return m;
}

template<class V>
bool in_range(const V& v, int32_t index)
{
  return index >= 0 && index < static_cast<int32_t>(v.size());
}

template<class V>
int index_of_id(const V& v, int32_t id, int32_t* index, const char* what)
{
  for (size_t k = 0; k < v.size(); ++k)
    if (v[k].id == id) {
      *index = static_cast<int32_t>(k);
      return 0;
    }
  return capi_fail(OPENMC_E_INVALID_ID, std::string("No ") + what + " exists with ID=" + std::to_string(id) + ".");
}

const char* filter_type_str(int type)
{
  switch (type) {
  case omc::FILTER_MESH: return "mesh";
  case omc::FILTER_ENERGY: return "energy";
  case omc::FILTER_PARTICLE: return "particle";
  case omc::FILTER_CELL: return "cell";
  default: return "material";
  }
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- run state
// src/initialize.cpp (openmc_master), src/state_point.cpp
// (openmc_is_statepoint_batch), src/settings.cpp:1285-1324 (batches),
// src/eigenvalue.cpp:420-440 (k-effective)
bool openmc_master() { return true; }

// the default statepoint batches: the last one (src/settings.cpp:1008-1017)
bool openmc_is_statepoint_batch()
{
  HModel* m = omc::capi_model();
  return m && current_batch == m->n_batches;
}

// ------------------------------------------------------------ model sizes
// src/cell.cpp:1820, src/material.cpp:1599, src/mesh.cpp:3900,
// src/nuclide.cpp:1105, src/tallies/filter.cpp:62 (0 before openmc_init)
int cells_size()
{
  HModel* m = omc::capi_model();
  return m ? static_cast<int>(m->cells.size()) : 0;
}

size_t n_materials()
{
  HModel* m = omc::capi_model();
  return m ? m->materials.size() : 0;
}

int n_meshes()
{
  HModel* m = omc::capi_model();
  return m ? static_cast<int>(m->meshes.size()) : 0;
}

size_t nuclides_size()
{
  HModel* m = omc::capi_model();
  return m ? m->nuclides.size() : 0;
}

size_t tally_filters_size()
{
  HModel* m = omc::capi_model();
  return m ? m->filters.size() : 0;
}

int openmc_get_n_batches(int* n_batches, bool get_max_batches)
{
  (void)get_max_batches;  // no triggers: n_batches == n_max_batches
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  *n_batches = m->n_batches;
  return 0;
}

int openmc_set_n_batches(int32_t n_batches, bool set_max_batches, bool add_statepoint_batch)
{
  (void)set_max_batches;
  (void)add_statepoint_batch;  // the statepoint is written at the last batch (the default statepoint batches)
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (m->n_inactive >= n_batches)
    return capi_fail(OPENMC_E_INVALID_ARGUMENT, "Number of active batches must be greater than zero.");
  m->n_batches = n_batches;
  return 0;
}

// -------------------------------------------------------- cells, materials
// src/cell.cpp (openmc_get_cell_index, openmc_cell_get_id,
// openmc_cell_get_translation, openmc_cell_get_name), src/material.cpp
// (openmc_get_material_index, openmc_material_get_id,
// openmc_material_get_name)
int openmc_get_cell_index(int32_t id, int32_t* index)
{
  int rc;
  HModel* m = model_or_fail(rc);
  return m ? index_of_id(m->cells, id, index, "cell") : rc;
}

int openmc_cell_get_id(int32_t index, int32_t* id)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->cells, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in cells array is out of bounds.");
  *id = m->cells[index].id;
  return 0;
}

int openmc_cell_get_translation(int32_t index, double xyz[])
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->cells, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in cells array is out of bounds.");
  for (int k = 0; k < 3; ++k) xyz[k] = m->cells[index].tr[k];
  return 0;
}

int openmc_cell_get_name(int32_t index, const char** name)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->cells, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in cells array is out of bounds.");
  *name = "";  // names are not kept by this library's model reader
  return 0;
}

int openmc_get_material_index(int32_t id, int32_t* index)
{
  int rc;
  HModel* m = model_or_fail(rc);
  return m ? index_of_id(m->materials, id, index, "material") : rc;
}

int openmc_material_get_id(int32_t index, int32_t* id)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->materials, index))
    return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in materials array is out of bounds.");
  *id = m->materials[index].id;
  return 0;
}

int openmc_material_get_name(int32_t index, const char** name)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->materials, index))
    return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in materials array is out of bounds.");
  *name = "";
  return 0;
}

// Atom densities [atom/b-cm] of the material's nuclides (borrowed) and the
// mass density [g/cm^3] = sum n_i awr_i m_n / N_A (src/material.cpp:
// 1389-1419, the sum of :456-466; neutron mass 1.00866491595 u, Avogadro
// 0.602214076e24 /mol).
int openmc_material_get_densities(int32_t index, const int** nuclides, const double** densities, int* n)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->materials, index))
    return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in materials array is out of bounds.");
  const omc::HMaterial& mat = m->materials[index];
  if (mat.nuclide.empty()) return capi_fail(OPENMC_E_ALLOCATE, "Material atom density array has not been allocated.");
  *nuclides = mat.nuclide.data();
  *densities = mat.atom_density.data();
  *n = static_cast<int>(mat.nuclide.size());
  return 0;
}

int openmc_material_get_density(int32_t index, double* density)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->materials, index))
    return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in materials array is out of bounds.");
  const omc::HMaterial& mat = m->materials[index];
  double rho = 0.0;
  for (size_t k = 0; k < mat.nuclide.size(); ++k)
    rho += mat.atom_density[k] * m->nuclides[mat.nuclide[k]].awr * 1.00866491595 / 0.602214076;
  *density = rho;
  return 0;
}

// Fill of a cell (src/cell.cpp openmc_cell_get_fill): type 0 material,
// 1 universe, 2 lattice (the reference's Fill enum), with a borrowed pointer
// to the one material, universe or lattice index.
int openmc_cell_get_fill(int32_t index, int* type, int32_t** indices, int32_t* n)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->cells, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in cells array is out of bounds.");
  omc::HCell& c = m->cells[index];
  *type = c.fill_type;
  *indices = &c.fill;
  *n = 1;
  return 0;
}

// Instances of a cell (src/geometry_aux.cpp count_cell_instances): one per
// path from the root universe through universe and lattice fills (a
// lattice's outer universe is not counted).
static void count_instances(const HModel& m, int univ, std::vector<int32_t>& n, int depth)
{
  if (univ < 0 || univ >= static_cast<int>(m.universes.size()) || depth > 64) return;
  for (int c : m.universes[univ]) {
    n[c] += 1;
    const omc::HCell& cell = m.cells[c];
    if (cell.fill_type == omc::FILL_UNIVERSE) {
      count_instances(m, cell.fill, n, depth + 1);
    } else if (cell.fill_type == omc::FILL_LATTICE && cell.fill >= 0 &&
               cell.fill < static_cast<int>(m.lattices.size())) {
      for (int u : m.lattices[cell.fill].univ) count_instances(m, u, n, depth + 1);
    }
  }
}

int openmc_cell_get_num_instances(int32_t index, int32_t* num_instances)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->cells, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in cells array is out of bounds.");
  std::vector<int32_t> n(m->cells.size(), 0);
  count_instances(*m, m->root_universe, n, 0);
  *num_instances = n[index];
  return 0;
}

// Bounding boxes (src/cell.cpp:1033-1076 Region::bounding_box, the surfaces'
// bounding_box(pos_side) in src/surface.cpp, Universe::bounding_box): the
// half-space of an axis plane bounds one axis, the inside of a cylinder its
// two transverse axes, the inside of a sphere all three; other half-spaces
// are unbounded.  Simple regions intersect their half-spaces; complex ones
// evaluate the postfix with union and intersection, a complemented
// sub-region counting as unbounded.
struct Box {
  double lo[3], hi[3];
  static Box inf()
  {
    const double I = std::numeric_limits<double>::infinity();
    return Box {{-I, -I, -I}, {I, I, I}};
  }
  static Box empty()
  {
    const double I = std::numeric_limits<double>::infinity();
    return Box {{I, I, I}, {-I, -I, -I}};
  }
  Box operator&(const Box& o) const
  {
    Box b;
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = std::max(lo[k], o.lo[k]);
      b.hi[k] = std::min(hi[k], o.hi[k]);
    }
    return b;
  }
  Box operator|(const Box& o) const
  {
    Box b;
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = std::min(lo[k], o.lo[k]);
      b.hi[k] = std::max(hi[k], o.hi[k]);
    }
    return b;
  }
};

static Box halfspace_box(const omc::HSurface& s, bool pos_side)
{
  Box b = Box::inf();
  if (s.type <= 2) {  // x-, y-, z-plane at c[0]
    (pos_side ? b.lo : b.hi)[s.type] = s.c[0];
  } else if (s.type <= 5 && !pos_side) {  // cylinder along x, y or z
    const int axis = s.type - 3;
    const int a = axis == 0 ? 1 : 0, c2 = axis == 2 ? 1 : 2;
    b.lo[a] = s.c[0] - s.c[2];
    b.hi[a] = s.c[0] + s.c[2];
    b.lo[c2] = s.c[1] - s.c[2];
    b.hi[c2] = s.c[1] + s.c[2];
  } else if (s.type == 6 && !pos_side) {  // sphere
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = s.c[k] - s.c[3];
      b.hi[k] = s.c[k] + s.c[3];
    }
  }
  return b;
}

static Box cell_box(const HModel& m, const omc::HCell& c)
{
  auto surf = [&](int32_t token) { return halfspace_box(m.surfaces[std::abs(token) - 1], token > 0); };
  if (c.simple) {
    Box b = Box::inf();
    for (int32_t t : c.expr) b = b & surf(t);
    return b;
  }
  std::vector<Box> st;
  for (int32_t t : c.expr) {
    if (t == omc::OP_UNION || t == omc::OP_INTERSECTION) {
      if (st.size() < 2) return Box::inf();
      Box r = st.back();
      st.pop_back();
      st.back() = t == omc::OP_UNION ? (st.back() | r) : (st.back() & r);
    } else if (t == omc::OP_COMPLEMENT) {
      if (st.empty()) return Box::inf();
      st.back() = Box::inf();
    } else {
      st.push_back(surf(t));
    }
  }
  return st.empty() ? Box::inf() : st.back();
}

int openmc_cell_bounding_box(const int32_t index, double* llc, double* urc)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->cells, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in cells array is out of bounds.");
  const Box b = cell_box(*m, m->cells[index]);
  for (int k = 0; k < 3; ++k) {
    llc[k] = b.lo[k];
    urc[k] = b.hi[k];
  }
  return 0;
}

int openmc_global_bounding_box(double* llc, double* urc)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  Box b = Box::empty();
  if (m->root_universe >= 0 && m->root_universe < static_cast<int>(m->universes.size()))
    for (int c : m->universes[m->root_universe]) b = b | cell_box(*m, m->cells[c]);
  for (int k = 0; k < 3; ++k) {
    llc[k] = b.lo[k];
    urc[k] = b.hi[k];
  }
  return 0;
}

// ----------------------------------------------------------------- nuclides
// src/nuclide.cpp (openmc_get_nuclide_index, openmc_nuclide_name)
int openmc_get_nuclide_index(const char name[], int* index)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  for (size_t k = 0; k < m->nuclides.size(); ++k)
    if (m->nuclides[k].name == name) {
      *index = static_cast<int>(k);
      return 0;
    }
  return capi_fail(OPENMC_E_DATA, std::string("No nuclide named '") + name + "' has been loaded.");
}

int openmc_nuclide_name(int index, const char** name)
{
  int rc;
  HModel* m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->nuclides, index))
    return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in nuclides array is out of bounds.");
  *name = m->nuclides[index].name.c_str();
  return 0;
}

// ------------------------------------------------------------------- meshes
// src/mesh.cpp (openmc_get_mesh_index, openmc_mesh_get_id,
// openmc_mesh_get_type :2285-2293, openmc_mesh_get_n_elements,
// openmc_mesh_bounding_box, openmc_regular_mesh_get_dimension :2508-2517,
// openmc_regular_mesh_get_params :2534-2555); every mesh here is regular
int openmc_get_mesh_index(int32_t id, int32_t* index)
{
  int rc;
  HModel* m = model_or_fail(rc);
  return m ? index_of_id(m->meshes, id, index, "mesh") : rc;
}

static int check_mesh(HModel*& m, int32_t index)
{
  int rc;
  m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->meshes, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in meshes array is out of bounds.");
  return 0;
}

int openmc_mesh_get_id(int32_t index, int32_t* id)
{
  HModel* m;
  if (int rc = check_mesh(m, index)) return rc;
  *id = m->meshes[index].id;
  return 0;
}

int openmc_mesh_get_type(int32_t index, char* type)
{
  HModel* m;
  if (int rc = check_mesh(m, index)) return rc;
  std::strcpy(type, "regular");
  return 0;
}

int openmc_mesh_get_n_elements(int32_t index, size_t* n)
{
  HModel* m;
  if (int rc = check_mesh(m, index)) return rc;
  *n = static_cast<size_t>(m->meshes[index].n_bins());
  return 0;
}

int openmc_mesh_bounding_box(int32_t index, double* ll, double* ur)
{
  HModel* m;
  if (int rc = check_mesh(m, index)) return rc;
  const omc::HMesh& h = m->meshes[index];
  for (int k = 0; k < 3; ++k) {
    const bool used = k < h.ndim;
    ll[k] = used ? h.ll[k] : -std::numeric_limits<double>::infinity();
    ur[k] = used ? h.ur[k] : std::numeric_limits<double>::infinity();
  }
  return 0;
}

int openmc_regular_mesh_get_dimension(int32_t index, int** dims, int* n)
{
  HModel* m;
  if (int rc = check_mesh(m, index)) return rc;
  *dims = m->meshes[index].shape;
  *n = m->meshes[index].ndim;
  return 0;
}

int openmc_regular_mesh_get_params(int32_t index, double** ll, double** ur, double** width, int* n)
{
  HModel* m;
  if (int rc = check_mesh(m, index)) return rc;
  omc::HMesh& h = m->meshes[index];
  *ll = h.ll;
  *ur = h.ur;
  *width = h.width;
  *n = h.ndim;
  return 0;
}

// ------------------------------------------------------------------ filters
// src/tallies/filter.cpp (openmc_get_filter_index, openmc_filter_get_id,
// openmc_filter_get_type :234-241, openmc_filter_get_num_bins :243-250),
// filter_energy.cpp (openmc_energy_filter_get_bins), filter_mesh.cpp
// (openmc_mesh_filter_get_mesh), filter_cell.cpp
// (openmc_cell_filter_get_bins), filter_material.cpp
// (openmc_material_filter_get_bins)
int openmc_get_filter_index(int32_t id, int32_t* index)
{
  int rc;
  HModel* m = model_or_fail(rc);
  return m ? index_of_id(m->filters, id, index, "filter") : rc;
}

static int check_filter(HModel*& m, int32_t index, int type = -1)
{
  int rc;
  m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->filters, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in filters array is out of bounds.");
  if (type >= 0 && m->filters[index].type != type)
    return capi_fail(OPENMC_E_INVALID_TYPE, std::string("Tried to get bins on a non-") + filter_type_str(type) +
                                                " filter.");
  return 0;
}

int openmc_filter_get_id(int32_t index, int32_t* id)
{
  HModel* m;
  if (int rc = check_filter(m, index)) return rc;
  *id = m->filters[index].id;
  return 0;
}

int openmc_filter_get_type(int32_t index, char* type)
{
  HModel* m;
  if (int rc = check_filter(m, index)) return rc;
  std::strcpy(type, filter_type_str(m->filters[index].type));
  return 0;
}

int openmc_filter_get_num_bins(int32_t index, int* n_bins)
{
  HModel* m;
  if (int rc = check_filter(m, index)) return rc;
  *n_bins = m->filters[index].nbins;
  return 0;
}

int openmc_energy_filter_get_bins(int32_t index, const double** energies, size_t* n)
{
  HModel* m;
  if (int rc = check_filter(m, index, omc::FILTER_ENERGY)) return rc;
  *energies = m->filters[index].bins.data();
  *n = m->filters[index].bins.size();
  return 0;
}

int openmc_mesh_filter_get_mesh(int32_t index, int32_t* index_mesh)
{
  HModel* m;
  if (int rc = check_filter(m, index, omc::FILTER_MESH)) return rc;
  *index_mesh = m->filters[index].mesh;
  return 0;
}

int openmc_cell_filter_get_bins(int32_t index, const int32_t** cells, int32_t* n)
{
  HModel* m;
  if (int rc = check_filter(m, index, omc::FILTER_CELL)) return rc;
  *cells = m->filters[index].ids.data();
  *n = static_cast<int32_t>(m->filters[index].ids.size());
  return 0;
}

int openmc_material_filter_get_bins(int32_t index, const int32_t** bins, size_t* n)
{
  HModel* m;
  if (int rc = check_filter(m, index, omc::FILTER_MATERIAL)) return rc;
  *bins = m->filters[index].ids.data();
  *n = m->filters[index].ids.size();
  return 0;
}

// Mesh filters here carry no translation; particle filters bin neutrons
// only (ParticleType::neutron = 0).
int openmc_mesh_filter_get_translation(int32_t index, double translation[3])
{
  HModel* m;
  if (int rc = check_filter(m, index, omc::FILTER_MESH)) return rc;
  translation[0] = translation[1] = translation[2] = 0.0;
  return 0;
}

int openmc_particle_filter_get_bins(int32_t idx, int bins[])
{
  HModel* m;
  if (int rc = check_filter(m, idx, omc::FILTER_PARTICLE)) return rc;
  for (int b = 0; b < m->filters[idx].nbins; ++b) bins[b] = 0;
  return 0;
}

// ------------------------------------------------------------------ tallies
// src/tallies/tally.cpp (openmc_tally_get_type, _get_estimator, _get_active,
// _get_writable, _get_multiply_density, _get_filters, _get_scores,
// _get_nuclides).  Every tally here is a volume tally, active, writable and
// multiplied by density, over the total of all nuclides; scores are
// reported with the reference's codes (include/openmc/constants.h:310-314:
// flux -1, total -2, absorption -5) and estimators with TallyEstimator
// (:299; track-length 1, collision 2).
static int check_tally(HModel*& m, int32_t index)
{
  int rc;
  m = model_or_fail(rc);
  if (!m) return rc;
  if (!in_range(m->tallies, index)) return capi_fail(OPENMC_E_OUT_OF_BOUNDS, "Index in tallies array is out of bounds.");
  return 0;
}

int openmc_tally_get_type(int32_t index, int32_t* type)
{
  HModel* m;
  if (int rc = check_tally(m, index)) return rc;
  *type = 0;  // TallyType::VOLUME
  return 0;
}

int openmc_tally_get_estimator(int32_t index, int* estimator)
{
  HModel* m;
  if (int rc = check_tally(m, index)) return rc;
  *estimator = m->tallies[index].estimator == omc::EST_COLLISION ? 2 : 1;
  return 0;
}

int openmc_tally_get_active(int32_t index, bool* active)
{
  HModel* m;
  if (int rc = check_tally(m, index)) return rc;
  *active = true;
  return 0;
}

int openmc_tally_get_writable(int32_t index, bool* writable)
{
  HModel* m;
  if (int rc = check_tally(m, index)) return rc;
  *writable = true;
  return 0;
}

int openmc_tally_get_multiply_density(int32_t index, bool* value)
{
  HModel* m;
  if (int rc = check_tally(m, index)) return rc;
  *value = true;
  return 0;
}

int openmc_tally_get_filters(int32_t index, const int32_t** indices, size_t* n)
{
  HModel* m;
  if (int rc = check_tally(m, index)) return rc;
  *indices = m->tallies[index].filters.data();
  *n = m->tallies[index].filters.size();
  return 0;
}

int openmc_tally_get_scores(int32_t index, int** scores, int* n)
{
  HModel* m;
  if (int rc = check_tally(m, index)) return rc;
  // the reference codes live as long as the tally (a borrowed pointer)
  static std::map<const omc::HTally*, std::vector<int>> codes;
  const omc::HTally& t = m->tallies[index];
  std::vector<int>& c = codes[&t];
  c.clear();
  for (int s : t.scores) c.push_back(s == omc::SCORE_FLUX ? -1 : (s == omc::SCORE_TOTAL ? -2 : -5));
  *scores = c.data();
  *n = static_cast<int>(c.size());
  return 0;
}

int openmc_tally_get_nuclides(int32_t index, int** nuclides, int* n)
{
  HModel* m;
  if (int rc = check_tally(m, index)) return rc;
  static int total = -1;  // the "total" nuclide bin
  *nuclides = &total;
  *n = 1;
  return 0;
}

}  // extern "C"
