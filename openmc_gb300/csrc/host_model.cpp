// Loading of OpenMC XML input and the nuclide library into HModel.
//
// Element names and meanings follow the reference readers:
//   materials   src/material.cpp (Material::Material, normalize_density :417-467)
//   geometry    src/surface.cpp, src/cell.cpp (Region::Region :556-683),
//               src/lattice.cpp:160-230 (RectLattice, universes top row first)
//   settings    src/settings.cpp (particles, batches, seed, event_based :1192,
//               log_grid_bins :607, weight windows :1201-1262, cutoff)
//   tallies     src/tallies/tally.cpp, filter_mesh.cpp, filter_energy.cpp
//   source      src/source.cpp (IndependentSource, constraints :94-150)
//   data        cross_sections.xml library (src/cross_sections.cpp:183-343);
//               nuclide payloads use this project's binary container because
//               neither machine has HDF5 (field list in openmc_gb300/data.py).
#include "host_model.h"

#include "h5lite.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <functional>
#include <limits>
#include <map>
#include <sstream>
#include <stdexcept>

#include "xml.h"

namespace omc {

namespace {

std::string read_file(const std::string& path)
{
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

bool file_exists(const std::string& p)
{
  std::ifstream f(p);
  return static_cast<bool>(f);
}

std::string dirname_of(const std::string& p)
{
  size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

std::string join(const std::string& dir, const std::string& f)
{
  if (!f.empty() && f[0] == '/') return f;
  return dir + "/" + f;
}

// src/nuclide.cpp:359-453 create_derived from the MT 2, 18 (may be empty) and
// 102 cross sections on the nuclide's grid
void derive_columns(HNuclide& nuc, std::vector<double> el, const std::vector<double>& fis,
                    const std::vector<double>& cap)
{
  const size_t G = nuc.energy.size();
  // the grid the lookups search: at least two points, positive, finite and
  // non-decreasing (repeated points are allowed, as in evaluated data)
  if (G < 2) throw std::runtime_error("nuclide " + nuc.name + ": energy grid of fewer than two points");
  for (size_t k = 0; k < G; ++k) {
    if (!(nuc.energy[k] > 0.0) || !std::isfinite(nuc.energy[k]) || (k > 0 && nuc.energy[k] < nuc.energy[k - 1]))
      throw std::runtime_error("nuclide " + nuc.name + ": energy grid not positive and ascending");
  }
  // src/nuclide.cpp:359-453: total and absorption start at zero; the
  // reactions are added in name (MT) order: MT 2 to total; MT 18 to total,
  // fission and absorption; MT 102 (disappearance) to total and absorption;
  // then nu_fission = nu(E) x fission per grid point (Polynomial, Horner in
  // increasing powers, src/endf.cpp:125-134)
  nuc.total.assign(G, 0.0);
  nuc.absorption.assign(G, 0.0);
  nuc.fission.assign(G, 0.0);
  nuc.nu_fission.assign(G, 0.0);
  for (size_t k = 0; k < G; ++k) nuc.total[k] += el[k];
  if (!fis.empty()) {
    for (size_t k = 0; k < G; ++k) {
      nuc.total[k] += fis[k];
      nuc.fission[k] += fis[k];
      nuc.absorption[k] += fis[k];
    }
  }
  for (size_t k = 0; k < G; ++k) {
    nuc.total[k] += cap[k];
    nuc.absorption[k] += cap[k];
  }
  if (!fis.empty()) {
    for (size_t k = 0; k < G; ++k) {
      double y = 0.0;
      for (int c = 1; c >= 0; --c) y = y * nuc.energy[k] + nuc.nu_c[c];
      nuc.nu_fission[k] = y * nuc.fission[k];
    }
  }
  nuc.elastic = std::move(el);
}

// One nuclide in OpenMC's incident-neutron HDF5 layout
// (docs/source/io_formats/nuclear_data.rst; src/nuclide.cpp:60-352 reads the
// same fields): atomic weight ratio, the one temperature's kT and energy
// grid, the MT 2 / 18 / 102 cross sections with threshold index 0 on that
// grid, and for MT 18 the prompt neutron product's Polynomial yield and
// uncorrelated Maxwell or Watt spectrum with constant parameters.
void read_nuclide_h5(const std::string& path, HNuclide& nuc)
{
  h5::File f(path);
  const h5::Node root = f.root();
  std::string gname = nuc.name;
  if (!root.has(gname)) {
    const auto names = root.children();
    if (names.size() != 1) throw std::runtime_error(path + ": no group for nuclide " + nuc.name);
    gname = names[0];
  }
  const h5::Node g = root.at(gname);
  nuc.awr = g.attr("atomic_weight_ratio").doubles().at(0);
  const auto temps = g.at("kTs").children();
  if (temps.size() != 1) throw std::runtime_error(path + ": one temperature per nuclide is supported");
  const std::string T = temps[0];
  nuc.kT = g.at("kTs/" + T).read().doubles().at(0);
  nuc.energy = g.at("energy/" + T).read().doubles();
  const size_t G = nuc.energy.size();
  std::vector<double> el, fis, cap;
  const h5::Node rxs = g.at("reactions");
  for (const std::string& name : rxs.children()) {
    if (name.rfind("reaction_", 0) != 0) continue;
    const h5::Node rx = rxs.at(name);
    const long long mt = rx.attr("mt").ints().at(0);
    if (rx.has_attr("redundant") && rx.attr("redundant").ints().at(0) != 0) continue;
    const h5::Node xs = rx.at(T + "/xs");
    const long long thr = xs.has_attr("threshold_idx") ? xs.attr("threshold_idx").ints().at(0) : 0;
    std::vector<double> v = xs.read().doubles();
    if (thr != 0 || v.size() != G) throw std::runtime_error(path + ": threshold reactions are not supported");
    if (mt == 2) {
      el = std::move(v);
    } else if (mt == 102) {
      cap = std::move(v);
    } else if (mt == 18) {
      fis = std::move(v);
      const h5::Node prod = rx.at("product_0");
      const std::vector<double> yc = prod.at("yield").read().doubles();
      if (yc.empty() || yc.size() > 2) throw std::runtime_error(path + ": fission yield must be a polynomial of degree <= 1");
      nuc.nu_c[0] = yc[0];
      nuc.nu_c[1] = yc.size() > 1 ? yc[1] : 0.0;
      const h5::Node en = prod.at("distribution_0/energy");
      const std::string type = en.attr("type").str();
      nuc.u = en.attr("u").doubles().at(0);
      // a constant Tabulated1D parameter: [[x...], [y...]] with equal y
      auto constant = [&](const char* ds) {
        const std::vector<double> t = en.at(ds).read().doubles();
        const size_t n = t.size() / 2;
        if (n == 0) throw std::runtime_error(path + ": empty spectrum parameter");
        for (size_t k = n; k < t.size(); ++k)
          if (t[k] != t[n]) throw std::runtime_error(path + ": energy-dependent spectrum parameters are not supported");
        return t[n];
      };
      if (type == "maxwell") {
        nuc.spectrum = 1;
        nuc.sp[0] = constant("theta");
      } else if (type == "watt") {
        nuc.spectrum = 2;
        nuc.sp[0] = constant("a");
        nuc.sp[1] = constant("b");
      } else {
        throw std::runtime_error(path + ": fission spectrum '" + type + "' is not supported");
      }
      nuc.fissionable = true;
    } else {
      throw std::runtime_error(path + ": only MT 2, MT 18 and MT 102 are supported");
    }
  }
  if (el.empty() || cap.empty()) throw std::runtime_error(path + ": needs MT 2 and MT 102");
  derive_columns(nuc, std::move(el), fis, cap);
}

void read_nuclide_file(const std::string& path, HNuclide& nuc)
{
  {
    std::ifstream probe(path, std::ios::binary);
    char sig[8] = {0};
    probe.read(sig, 8);
    if (std::memcmp(sig, "\x89HDF\r\n\x1a\n", 8) == 0) {
      read_nuclide_h5(path, nuc);
      return;
    }
  }
  std::string b = read_file(path);
  if (b.size() < 16 || std::memcmp(b.data(), "OMCGBNUC", 8) != 0)
    throw std::runtime_error(path + ": not a nuclide file");
  size_t off = 8;
  // every read checked against the file's size (a truncated file is an error)
  auto need = [&](size_t n) {
    if (n > b.size() - off) throw std::runtime_error(path + ": truncated nuclide file");
  };
  auto u32 = [&](void) {
    need(4);
    uint32_t v;
    std::memcpy(&v, b.data() + off, 4);
    off += 4;
    return v;
  };
  auto f64 = [&](void) {
    need(8);
    double v;
    std::memcpy(&v, b.data() + off, 8);
    off += 8;
    return v;
  };
  uint32_t version = u32();
  if (version != 1 && version != 2) throw std::runtime_error(path + ": unsupported nuclide file version");
  uint32_t nl = u32();
  need(nl);
  off += nl;
  f64();  // A
  nuc.awr = f64();
  nuc.kT = f64();
  uint32_t G = u32();
  uint32_t nrx = u32();
  need(8 * size_t(G));
  nuc.energy.resize(G);
  std::memcpy(nuc.energy.data(), b.data() + off, 8 * size_t(G));
  off += 8 * size_t(G);
  std::vector<double> el, fis, cap;
  for (uint32_t r = 0; r < nrx; ++r) {
    uint32_t mt = u32(), thr = u32(), n = u32();
    if (thr != 0 || n != G) throw std::runtime_error(path + ": threshold reactions are not supported");
    need(8 * size_t(n));
    std::vector<double> xs(n);
    std::memcpy(xs.data(), b.data() + off, 8 * size_t(n));
    off += 8 * size_t(n);
    if (mt == 2) el = std::move(xs);
    else if (mt == 18) fis = std::move(xs);
    else if (mt == 102) cap = std::move(xs);
    else throw std::runtime_error(path + ": only MT 2, MT 18 and MT 102 are supported");
  }
  if (el.empty() || cap.empty()) throw std::runtime_error(path + ": needs MT 2 and MT 102");
  if (version >= 2 && u32() != 0) {
    nuc.fissionable = true;
    nuc.nu_c[0] = f64();
    nuc.nu_c[1] = f64();
    nuc.spectrum = static_cast<int>(u32());
    nuc.sp[0] = f64();
    nuc.sp[1] = f64();
    nuc.u = f64();
    if (nuc.spectrum != 1 && nuc.spectrum != 2) throw std::runtime_error(path + ": unknown fission spectrum");
  }
  if (nuc.fissionable != !fis.empty()) throw std::runtime_error(path + ": MT 18 needs its fission neutron data");
  derive_columns(nuc, std::move(el), fis, cap);
}

// Region string -> tokens (src/cell.cpp:556-683).  Simple regions keep the
// surface tokens only; regions with a union or complement become postfix.
void parse_region(const std::string& spec, const std::map<int, int>& surf_index, HCell& c)
{
  std::vector<int32_t> t;
  for (size_t i = 0; i < spec.size();) {
    char ch = spec[i];
    if (ch == '(') { t.push_back(OP_LEFT_PAREN); ++i; }
    else if (ch == ')') { t.push_back(OP_RIGHT_PAREN); ++i; }
    else if (ch == '|') { t.push_back(OP_UNION); ++i; }
    else if (ch == '~') { t.push_back(OP_COMPLEMENT); ++i; }
    else if (ch == '-' || ch == '+' || isdigit(static_cast<unsigned char>(ch))) {
      size_t j = i + 1;
      while (j < spec.size() && isdigit(static_cast<unsigned char>(spec[j]))) ++j;
      int v = std::stoi(spec.substr(i, j - i));
      auto it = surf_index.find(std::abs(v));
      if (it == surf_index.end())
        throw std::runtime_error("Invalid surface ID " + std::to_string(std::abs(v)) +
                                 " specified in region for cell " + std::to_string(c.id) + ".");
      int idx = it->second + 1;
      t.push_back(v > 0 ? idx : -idx);
      i = j;
    } else if (isspace(static_cast<unsigned char>(ch))) {
      ++i;
    } else {
      throw std::runtime_error(std::string("Region specification contains invalid character, \"") + ch + "\"");
    }
  }
  std::vector<int32_t> e;
  for (size_t k = 0; k < t.size(); ++k) {
    e.push_back(t[k]);
    if (k + 1 < t.size()) {
      bool left = t[k] < OP_UNION || t[k] == OP_RIGHT_PAREN;
      bool right = t[k + 1] < OP_UNION || t[k + 1] == OP_LEFT_PAREN || t[k + 1] == OP_COMPLEMENT;
      if (left && right) e.push_back(OP_INTERSECTION);
    }
  }
  bool simple = std::find(e.begin(), e.end(), OP_UNION) == e.end() &&
                std::find(e.begin(), e.end(), OP_COMPLEMENT) == e.end();
  c.simple = simple;
  if (simple) {
    for (int32_t v : e)
      if (v < OP_UNION) c.expr.push_back(v);
    return;
  }
  auto prec = [](int32_t op) { return op == OP_COMPLEMENT ? 3 : (op == OP_INTERSECTION ? 2 : 1); };
  std::vector<int32_t> st;
  for (int32_t v : e) {
    if (v < OP_UNION) {
      c.expr.push_back(v);
    } else if (v == OP_LEFT_PAREN || v == OP_COMPLEMENT) {
      st.push_back(v);
    } else if (v == OP_RIGHT_PAREN) {
      while (!st.empty() && st.back() != OP_LEFT_PAREN) { c.expr.push_back(st.back()); st.pop_back(); }
      if (st.empty()) throw std::runtime_error("unbalanced parentheses in region of cell " + std::to_string(c.id));
      st.pop_back();
      if (!st.empty() && st.back() == OP_COMPLEMENT) { c.expr.push_back(st.back()); st.pop_back(); }
    } else {
      while (!st.empty() && st.back() != OP_LEFT_PAREN && prec(st.back()) >= prec(v)) {
        c.expr.push_back(st.back());
        st.pop_back();
      }
      st.push_back(v);
    }
  }
  while (!st.empty()) { c.expr.push_back(st.back()); st.pop_back(); }
}

int surface_type(const std::string& t)
{
  if (t == "x-plane") return SURF_XPLANE;
  if (t == "y-plane") return SURF_YPLANE;
  if (t == "z-plane") return SURF_ZPLANE;
  if (t == "x-cylinder") return SURF_XCYL;
  if (t == "y-cylinder") return SURF_YCYL;
  if (t == "z-cylinder") return SURF_ZCYL;
  if (t == "sphere") return SURF_SPHERE;
  throw std::runtime_error("surface type '" + t + "' is not supported by the GPU transport path");
}

void read_mesh(const XmlNode* el, std::vector<HMesh>& meshes)
{
  HMesh m;
  m.id = std::stoi(el->value("id"));
  std::string type = el->value_or("type", "regular");
  if (type != "regular") throw std::runtime_error("only regular meshes are supported (mesh " + std::to_string(m.id) + ")");
  for (const auto& e : meshes)
    if (e.id == m.id) throw std::runtime_error("Two or more meshes use the same unique ID: " + std::to_string(m.id));
  auto dim = split_ints(el->value("dimension"));
  auto ll = split_doubles(el->value("lower_left"));
  m.ndim = static_cast<int>(dim.size());
  if (m.ndim < 1 || m.ndim > 3 || ll.size() != dim.size())
    throw std::runtime_error("mesh " + std::to_string(m.id) + ": inconsistent dimensions");
  for (int i = 0; i < 3; ++i) {
    m.shape[i] = i < m.ndim ? static_cast<int>(dim[i]) : 1;
    m.ll[i] = i < m.ndim ? ll[i] : 0.0;
    m.ur[i] = 1.0;
    m.width[i] = 1.0;
  }
  // src/mesh.cpp:1183-1246 set_grid
  if (el->has("width")) {
    auto w = split_doubles(el->value("width"));
    for (int i = 0; i < m.ndim; ++i) {
      m.width[i] = w[i];
      m.ur[i] = m.ll[i] + m.shape[i] * w[i];
    }
  } else {
    auto ur = split_doubles(el->value("upper_right"));
    for (int i = 0; i < m.ndim; ++i) {
      m.ur[i] = ur[i];
      m.width[i] = (ur[i] - m.ll[i]) / m.shape[i];
    }
  }
  for (int i = 0; i < m.ndim; ++i)
    if (m.shape[i] <= 0) throw std::runtime_error("All entries for a regular mesh dimensions must be positive.");
  meshes.push_back(m);
}

int mesh_index(const HModel& m, int id)
{
  for (size_t k = 0; k < m.meshes.size(); ++k)
    if (m.meshes[k].id == id) return static_cast<int>(k);
  throw std::runtime_error("mesh " + std::to_string(id) + " not found");
}

}  // namespace

void load_model(const std::string& path_in, HModel& m)
{
  std::string dir = path_in.empty() ? std::string(".") : path_in;
  std::string model_path;
  if (dir.size() > 4 && dir.substr(dir.size() - 4) == ".xml") {
    model_path = dir;
    dir = dirname_of(dir);
  } else {
    model_path = join(dir, "model.xml");
  }
  std::unique_ptr<XmlNode> model_doc, mats_doc, geom_doc, set_doc, tal_doc;
  const XmlNode *mats, *geom, *set, *tal = nullptr;
  std::string model_src;
  if (file_exists(model_path)) {
    model_src = read_file(model_path);
    model_doc = XmlParser(model_src).parse();
    mats = model_doc->child("materials");
    geom = model_doc->child("geometry");
    set = model_doc->child("settings");
    tal = model_doc->child("tallies");
  } else {
    static thread_local std::string a, b, c, d;
    a = read_file(join(dir, "materials.xml"));
    b = read_file(join(dir, "geometry.xml"));
    c = read_file(join(dir, "settings.xml"));
    mats_doc = XmlParser(a).parse();
    geom_doc = XmlParser(b).parse();
    set_doc = XmlParser(c).parse();
    mats = mats_doc.get();
    geom = geom_doc.get();
    set = set_doc.get();
    if (file_exists(join(dir, "tallies.xml"))) {
      d = read_file(join(dir, "tallies.xml"));
      tal_doc = XmlParser(d).parse();
      tal = tal_doc.get();
    }
  }
  if (!mats || !geom || !set) throw std::runtime_error("model needs <materials>, <geometry> and <settings>");

  // ------------------------------------------------------- cross sections
  std::string xs_path;
  if (mats->child("cross_sections")) xs_path = XmlNode::trim(mats->child("cross_sections")->text);
  else if (const char* env = std::getenv("OPENMC_CROSS_SECTIONS")) xs_path = env;
  else throw std::runtime_error("No cross_sections.xml file was specified in materials.xml or in the "
                                "OPENMC_CROSS_SECTIONS environment variable.");
  xs_path = join(dir, xs_path);
  std::string xs_src = read_file(xs_path);
  auto xs_doc = XmlParser(xs_src).parse();
  std::map<std::string, std::string> library;
  for (const XmlNode* lib : xs_doc->all("library")) {
    if (lib->value_or("type", "neutron") != "neutron") continue;
    std::string p = join(dirname_of(xs_path), lib->value("path"));
    for (const auto& name : split_words(lib->value("materials"))) library[name] = p;
  }

  // ------------------------------------------------------------- materials
  std::vector<std::string> nuc_names;
  for (const XmlNode* me : mats->all("material")) {
    HMaterial mat;
    mat.id = std::stoi(me->value("id"));
    const XmlNode* d = me->child("density");
    if (!d) throw std::runtime_error("material " + std::to_string(mat.id) + " has no density");
    std::string units = d->value_or("units", "");
    double sum_ao = 0.0;
    for (const XmlNode* ne : me->all("nuclide")) {
      std::string name = ne->value("name");
      if (!ne->has("ao")) throw std::runtime_error("material " + std::to_string(mat.id) + ": only 'ao' fractions are supported");
      auto it = std::find(nuc_names.begin(), nuc_names.end(), name);
      int idx;
      if (it == nuc_names.end()) {
        idx = static_cast<int>(nuc_names.size());
        nuc_names.push_back(name);
      } else {
        idx = static_cast<int>(it - nuc_names.begin());
      }
      double ao = std::stod(ne->value("ao"));
      mat.nuclide.push_back(idx);
      mat.atom_density.push_back(ao);
      sum_ao += ao;
    }
    if (mat.nuclide.empty()) throw std::runtime_error("material " + std::to_string(mat.id) + " has no nuclides");
    double density;
    if (units == "sum") density = sum_ao;
    else if (units == "atom/b-cm") density = std::stod(d->value("value"));
    else throw std::runtime_error("material " + std::to_string(mat.id) + ": density units '" + units +
                                  "' are not supported (use atom/b-cm or sum)");
    // normalize_density (src/material.cpp:417-467) for atom percents
    double s = 0.0;
    for (double v : mat.atom_density) s += v;
    for (double& v : mat.atom_density) v /= s;
    for (double& v : mat.atom_density) v *= density;
    m.materials.push_back(std::move(mat));
  }
  for (const auto& name : nuc_names) {
    auto it = library.find(name);
    if (it == library.end()) throw std::runtime_error("Could not find nuclide " + name + " in cross_sections data file!");
    HNuclide nuc;
    nuc.name = name;
    read_nuclide_file(it->second, nuc);
    m.nuclides.push_back(std::move(nuc));
  }

  // -------------------------------------------------------------- geometry
  std::map<int, int> surf_index;
  for (const XmlNode* se : geom->all("surface")) {
    HSurface s {};
    s.id = std::stoi(se->value("id"));
    s.type = surface_type(se->value("type"));
    auto c = split_doubles(se->value("coeffs"));
    for (size_t k = 0; k < 4; ++k) s.c[k] = k < c.size() ? c[k] : 0.0;
    std::string bc = se->value_or("boundary", "transmission");
    if (bc == "transmission") s.bc = BC_TRANSMIT;
    else if (bc == "vacuum") s.bc = BC_VACUUM;
    else if (bc == "reflective") s.bc = BC_REFLECT;
    else throw std::runtime_error("boundary condition '" + bc + "' is not supported");
    surf_index[s.id] = static_cast<int>(m.surfaces.size());
    m.surfaces.push_back(s);
  }
  auto cell_nodes = geom->all("cell");
  auto lat_nodes = geom->all("lattice");
  std::map<int, int> univ_index, lat_index, mat_index;
  for (size_t k = 0; k < m.materials.size(); ++k) mat_index[m.materials[k].id] = static_cast<int>(k);
  for (const XmlNode* ce : cell_nodes) {
    int u = std::stoi(ce->value_or("universe", "0"));
    if (!univ_index.count(u)) {
      univ_index[u] = static_cast<int>(m.univ_ids.size());
      m.univ_ids.push_back(u);
    }
  }
  for (size_t k = 0; k < lat_nodes.size(); ++k) lat_index[std::stoi(lat_nodes[k]->value("id"))] = static_cast<int>(k);
  std::vector<int> filled;
  for (const XmlNode* ce : cell_nodes) {
    HCell c {};
    c.id = std::stoi(ce->value("id"));
    c.universe = univ_index[std::stoi(ce->value_or("universe", "0"))];
    if (ce->has("fill")) {
      int f = std::stoi(ce->value("fill"));
      filled.push_back(f);
      if (lat_index.count(f)) {
        c.fill_type = FILL_LATTICE;
        c.fill = lat_index[f];
      } else if (univ_index.count(f)) {
        c.fill_type = FILL_UNIVERSE;
        c.fill = univ_index[f];
      } else {
        throw std::runtime_error("cell " + std::to_string(c.id) + " is filled with unknown universe " + std::to_string(f));
      }
    } else {
      c.fill_type = FILL_MATERIAL;
      std::string mat = ce->value_or("material", "void");
      if (split_words(mat).size() > 1) throw std::runtime_error("distributed materials are not supported");
      if (mat == "void") c.fill = -1;
      else {
        int id = std::stoi(mat);
        if (!mat_index.count(id)) throw std::runtime_error("cell " + std::to_string(c.id) + ": unknown material " + mat);
        c.fill = mat_index[id];
      }
    }
    parse_region(ce->value_or("region", ""), surf_index, c);
    std::vector<double> tr = ce->has("translation") ? split_doubles(ce->value("translation")) : std::vector<double> {0, 0, 0};
    for (int k = 0; k < 3; ++k) c.tr[k] = tr[k];
    if (ce->has("rotation")) throw std::runtime_error("cell rotations are not supported");
    m.cells.push_back(std::move(c));
  }
  m.universes.assign(m.univ_ids.size(), {});
  for (size_t k = 0; k < m.cells.size(); ++k) m.universes[m.cells[k].universe].push_back(static_cast<int>(k));
  for (const XmlNode* le : lat_nodes) {
    HLattice lat {};
    lat.id = std::stoi(le->value("id"));
    auto dim = split_ints(le->value("dimension"));
    lat.is3d = dim.size() == 3;
    for (int i = 0; i < 3; ++i) lat.n[i] = i < static_cast<int>(dim.size()) ? static_cast<int>(dim[i]) : 1;
    auto ll = split_doubles(le->value("lower_left"));
    auto pitch = split_doubles(le->value("pitch"));
    if (ll.size() != dim.size() || pitch.size() != dim.size())
      throw std::runtime_error("lattice " + std::to_string(lat.id) + ": inconsistent dimensions");
    for (int i = 0; i < 3; ++i) {
      lat.ll[i] = i < static_cast<int>(ll.size()) ? ll[i] : 0.0;
      lat.pitch[i] = i < static_cast<int>(pitch.size()) ? pitch[i] : 0.0;
    }
    auto words = split_ints(le->value("universes"));
    int total = lat.n[0] * lat.n[1] * lat.n[2];
    if (static_cast<int>(words.size()) != total)
      throw std::runtime_error("Expected " + std::to_string(total) + " universes for lattice " + std::to_string(lat.id));
    lat.univ.assign(total, -1);
    for (int iz = 0; iz < lat.n[2]; iz++)
      for (int iy = lat.n[1] - 1; iy > -1; iy--)
        for (int ix = 0; ix < lat.n[0]; ix++) {
          int i1 = lat.n[0] * lat.n[1] * iz + lat.n[0] * (lat.n[1] - iy - 1) + ix;
          int i2 = lat.n[0] * lat.n[1] * iz + lat.n[0] * iy + ix;
          int uid = static_cast<int>(words[i2]);
          if (!univ_index.count(uid)) throw std::runtime_error("lattice " + std::to_string(lat.id) + ": unknown universe " + std::to_string(uid));
          lat.univ[i1] = univ_index[uid];
          filled.push_back(uid);
        }
    lat.outer = -1;
    if (le->has("outer")) {
      int o = std::stoi(le->value("outer"));
      filled.push_back(o);
      lat.outer = univ_index.at(o);
    }
    m.lattices.push_back(std::move(lat));
  }
  std::vector<int> roots;
  for (int u : m.univ_ids)
    if (std::find(filled.begin(), filled.end(), u) == filled.end()) roots.push_back(u);
  if (roots.size() != 1) throw std::runtime_error("could not determine a unique root universe");
  m.root_universe = univ_index[roots[0]];

  // -------------------------------------------------------------- settings
  std::string mode = XmlNode::trim(set->value_or("run_mode", "fixed source"));
  if (mode != "fixed source" && mode != "eigenvalue")
    throw std::runtime_error("run mode '" + mode + "' is not supported (fixed source and eigenvalue)");
  m.eigenvalue = mode == "eigenvalue";
  if (std::stoi(set->value_or("generations_per_batch", "1")) != 1)
    throw std::runtime_error("one generation per batch is supported");
  m.n_particles = std::stoll(set->value("particles"));
  m.n_batches = std::stoi(set->value("batches"));
  m.n_inactive = std::stoi(set->value_or("inactive", "0"));
  m.seed = std::stoll(set->value_or("seed", "1"));
  if (set->has("stride")) m.stride = std::stoull(set->value("stride"));
  m.n_log_bins = std::stoi(set->value_or("log_grid_bins", "8000"));
  if (m.n_log_bins < 1) throw std::runtime_error("Number of bins for logarithmic grid must be greater than zero.");
  m.event_based = XmlNode::trim(set->value_or("event_based", "false")) == "true";
  if (const XmlNode* out = set->child("output")) {
    if (out->has("tallies")) m.output_tallies = XmlNode::trim(out->value("tallies")) == "true";
    if (out->has("path")) m.path_output = XmlNode::trim(out->value("path"));
  }
  if (m.path_output.empty()) m.path_output = dir;
  if (set->has("max_particles_in_flight")) m.max_particles_in_flight = std::stoll(set->value("max_particles_in_flight"));
  if (set->has("max_history_splits")) m.max_history_splits = std::stoll(set->value("max_history_splits"));
  if (set->has("max_particle_events")) m.max_particle_events = std::stoi(set->value("max_particle_events"));
  if (set->has("max_lost_particles")) m.max_lost_particles = std::stoi(set->value("max_lost_particles"));
  if (set->has("rel_max_lost_particles")) m.rel_max_lost_particles = std::stod(set->value("rel_max_lost_particles"));
  if (const XmlNode* co = set->child("cutoff")) {
    if (co->has("energy_neutron")) m.energy_cutoff = std::stod(co->value("energy_neutron"));
    // src/settings.cpp:723-732; only neutrons are transported here, so the
    // other particles' time cutoffs have nothing to act on
    if (co->has("time_neutron")) m.time_cutoff = std::stod(co->value("time_neutron"));
    if (co->has("survival_biasing")) throw std::runtime_error("survival biasing is not supported");
  }
  if (set->has("survival_biasing") && XmlNode::trim(set->value("survival_biasing")) == "true")
    throw std::runtime_error("survival biasing is not supported");
  if (set->has("gb300_xs_precision")) {
    std::string p = set->value("gb300_xs_precision");
    m.xs_precision = (p == "fp32" || p == "32") ? 32 : 64;
  }
  for (const XmlNode* me : set->all("mesh")) read_mesh(me, m.meshes);

  // source
  auto srcs = set->all("source");
  if (srcs.size() != 1) throw std::runtime_error("exactly one <source> is supported");
  const XmlNode* src = srcs[0];
  std::string st = src->value_or("type", "independent");
  if (st != "independent") throw std::runtime_error("source type '" + st + "' is not supported");
  if (src->has("strength")) m.source.strength = std::stod(src->value("strength"));
  if (const XmlNode* sp = src->child("space")) {
    std::string t = sp->value_or("type", "point");
    if (t == "point") m.source.sp_type = 0;
    else if (t == "box") m.source.sp_type = 1;
    else throw std::runtime_error("spatial distribution '" + t + "' is not supported");
    m.source.sp = split_doubles(sp->value("parameters"));
    if (m.source.sp.size() != (m.source.sp_type == 0 ? 3u : 6u))
      throw std::runtime_error("spatial distribution has the wrong number of parameters");
  } else {
    m.source.sp = {0, 0, 0};
  }
  if (const XmlNode* an = src->child("angle")) {
    std::string t = an->value_or("type", "isotropic");
    if (t == "isotropic") m.source.an_type = 0;
    else if (t == "monodirectional") {
      m.source.an_type = 1;
      auto u = split_doubles(an->value("reference_uvw"));
      for (int k = 0; k < 3; ++k) m.source.uref[k] = u[k];
    } else throw std::runtime_error("angular distribution '" + t + "' is not supported");
  }
  if (const XmlNode* en = src->child("energy")) {
    std::string t = en->value_or("type", "discrete");
    if (t == "discrete") m.source.en_type = 0;
    else if (t == "maxwell") m.source.en_type = 1;
    else throw std::runtime_error("energy distribution '" + t + "' is not supported");
    m.source.en = split_doubles(en->value("parameters"));
  } else {
    throw std::runtime_error("the source needs an energy distribution");
  }
  const XmlNode* cons = src->child("constraints") ? src->child("constraints") : src;
  if (cons->has("domain_type")) {
    std::string t = cons->value("domain_type");
    m.source.dom_type = t == "cell" ? 0 : (t == "material" ? 1 : 2);
    for (auto v : split_ints(cons->value("domain_ids"))) m.source.dom_ids.push_back(static_cast<int>(v));
  }

  // weight windows
  for (const XmlNode* we : set->all("weight_windows")) {
    HWeightWindows w;
    w.id = std::stoi(we->value_or("id", "1"));
    w.mesh = mesh_index(m, std::stoi(we->value("mesh")));
    if (we->value_or("particle_type", "neutron") != "neutron") continue;
    w.ebounds = split_doubles(we->value("energy_bounds"));
    w.lower = split_doubles(we->value("lower_ww_bounds"));
    w.upper = split_doubles(we->value("upper_ww_bounds"));
    if (we->has("survival_ratio")) w.survival_ratio = std::stod(we->value("survival_ratio"));
    if (we->has("max_lower_bound_ratio")) w.max_lb_ratio = std::stod(we->value("max_lower_bound_ratio"));
    if (we->has("max_split")) w.max_split = std::stoi(we->value("max_split"));
    if (we->has("weight_cutoff")) w.weight_cutoff = std::stod(we->value("weight_cutoff"));
    size_t n = (w.ebounds.size() - 1) * static_cast<size_t>(m.meshes[w.mesh].n_bins());
    if (w.lower.size() != n || w.upper.size() != n)
      throw std::runtime_error("weight windows " + std::to_string(w.id) + ": bounds have the wrong size");
    m.weight_windows.push_back(std::move(w));
  }
  m.ww_on = !m.weight_windows.empty();
  if (set->has("weight_windows_on")) m.ww_on = XmlNode::trim(set->value("weight_windows_on")) == "true";
  if (const XmlNode* gens = set->child("weight_window_generators")) {
    for (const XmlNode* ge : gens->all("weight_windows_generator")) {
      HWWGenerator g;
      g.mesh = mesh_index(m, std::stoi(ge->value("mesh")));
      if (ge->has("energy_bounds")) g.ebounds = split_doubles(ge->value("energy_bounds"));
      if (ge->has("max_realizations")) g.max_realizations = std::stoi(ge->value("max_realizations"));
      if (ge->has("update_interval")) g.update_interval = std::stoi(ge->value("update_interval"));
      if (ge->has("on_the_fly")) g.on_the_fly = XmlNode::trim(ge->value("on_the_fly")) == "true";
      g.method = ge->value_or("method", "magic");
      if (g.method != "magic") throw std::runtime_error("only MAGIC weight-window generation is supported");
      if (const XmlNode* up = ge->child("update_parameters")) {
        g.value = up->value_or("value", "mean");
        g.threshold = std::stod(up->value_or("threshold", "1.0"));
        g.ratio = std::stod(up->value_or("ratio", "5.0"));
      }
      m.ww_generators.push_back(std::move(g));
    }
  }

  // ---------------------------------------------------------------- tallies
  if (tal) {
    for (const XmlNode* me : tal->all("mesh")) read_mesh(me, m.meshes);
    std::map<int, int> filt_index;
    for (const XmlNode* fe : tal->all("filter")) {
      HFilter f {};
      f.id = std::stoi(fe->value("id"));
      std::string t = fe->value("type");
      std::string bins = fe->value("bins");
      if (t == "mesh") {
        f.type = FILTER_MESH;
        f.mesh = mesh_index(m, std::stoi(bins));
        f.nbins = static_cast<int>(m.meshes[f.mesh].n_bins());
      } else if (t == "energy") {
        f.type = FILTER_ENERGY;
        f.mesh = -1;
        f.bins = split_doubles(bins);
        if (f.bins.size() < 2) throw std::runtime_error("energy filter needs two or more bin edges");
        f.nbins = static_cast<int>(f.bins.size()) - 1;
      } else if (t == "particle") {
        if (split_words(bins) != std::vector<std::string> {"neutron"})
          throw std::runtime_error("particle filters other than 'neutron' are not supported");
        f.type = FILTER_PARTICLE;
        f.mesh = -1;
        f.nbins = 1;
      } else if (t == "cell" || t == "material") {
        // src/tallies/filter_cell.cpp:48-58, filter_material.cpp:47-55
        f.type = t == "cell" ? FILTER_CELL : FILTER_MATERIAL;
        f.mesh = -1;
        for (auto id : split_ints(bins)) {
          int found = -1;
          if (f.type == FILTER_CELL) {
            for (size_t k = 0; k < m.cells.size(); ++k)
              if (m.cells[k].id == static_cast<int>(id)) found = static_cast<int>(k);
          } else {
            for (size_t k = 0; k < m.materials.size(); ++k)
              if (m.materials[k].id == static_cast<int>(id)) found = static_cast<int>(k);
          }
          if (found < 0) throw std::runtime_error(t + " filter " + std::to_string(f.id) + ": unknown id " + std::to_string(id));
          f.ids.push_back(found);
        }
        f.nbins = static_cast<int>(f.ids.size());
        if (f.nbins == 0) throw std::runtime_error(t + " filter " + std::to_string(f.id) + " has no bins");
      } else {
        throw std::runtime_error("filter type '" + t + "' is not supported by the GPU transport path");
      }
      filt_index[f.id] = static_cast<int>(m.filters.size());
      m.filters.push_back(std::move(f));
    }
    for (const XmlNode* te : tal->all("tally")) {
      HTally t;
      t.id = std::stoi(te->value("id"));
      t.name = te->value_or("name", "");
      if (te->has("filters"))
        for (auto fid : split_ints(te->value("filters"))) {
          if (!filt_index.count(static_cast<int>(fid))) throw std::runtime_error("tally " + std::to_string(t.id) + ": unknown filter");
          t.filters.push_back(filt_index[static_cast<int>(fid)]);
        }
      std::string est = XmlNode::trim(te->value_or("estimator", "tracklength"));
      if (est == "tracklength") t.estimator = EST_TRACKLENGTH;
      else if (est == "collision") t.estimator = EST_COLLISION;
      else throw std::runtime_error("only track-length and collision estimators are supported");
      if (te->has("nuclides") && XmlNode::trim(te->value("nuclides")) != "total")
        throw std::runtime_error("nuclide bins other than 'total' are not supported");
      for (const auto& s : split_words(te->value("scores"))) {
        if (s == "flux") t.scores.push_back(SCORE_FLUX);
        else if (s == "total") t.scores.push_back(SCORE_TOTAL);
        else if (s == "absorption") t.scores.push_back(SCORE_ABSORPTION);
        else throw std::runtime_error("score '" + s + "' is not supported by the GPU transport path");
      }
      int n_mesh = 0;
      for (int f : t.filters) n_mesh += m.filters[f].type == FILTER_MESH;
      if (n_mesh > 1) throw std::runtime_error("a tally may hold at most one mesh filter");
      int n_cell = 0;
      for (int f : t.filters) n_cell += m.filters[f].type == FILTER_CELL;
      if (n_cell > 1) throw std::runtime_error("a tally may hold at most one cell filter");
      if (t.filters.size() > 3) throw std::runtime_error("a tally may hold at most three filters");
      m.tallies.push_back(std::move(t));
    }
  }
}

void finalize_model(HModel& m)
{
  // src/simulation.cpp:682-761 initialize_data
  m.energy_min = 0.0;
  m.energy_max = std::numeric_limits<double>::max();
  for (const auto& n : m.nuclides) {
    m.energy_min = std::max(m.energy_min, n.energy.front());
    m.energy_max = std::min(m.energy_max, n.energy.back());
  }
  const int M = m.n_log_bins;
  // src/nuclide.cpp:502-533 init_grid (umesh points start + step*k, the last
  // one exactly M*spacing)
  for (auto& n : m.nuclides) {
    double spacing = std::log(m.energy_max / m.energy_min) / M;
    double stop = M * spacing;
    double step = stop / M;
    n.grid_index.assign(M + 1, 0);
    int j = 0;
    int G = static_cast<int>(n.energy.size());
    for (int k = 0; k <= M; ++k) {
      double umesh = (k == M) ? stop : 0.0 + step * k;
      while (std::log(n.energy[j + 1] / m.energy_min) <= umesh) {
        if (j + 2 == G) break;
        ++j;
      }
      n.grid_index[k] = j;
    }
  }
  m.log_spacing = std::log(m.energy_max / m.energy_min) / M;

  // tally strides (last filter stride 1) and result arrays
  for (auto& t : m.tallies) {
    t.strides.assign(t.filters.size(), 1);
    int64_t stride = 1;
    for (int i = static_cast<int>(t.filters.size()) - 1; i >= 0; --i) {
      t.strides[i] = static_cast<int>(stride);
      stride *= m.filters[t.filters[i]].nbins;
    }
    t.n_filter_bins = stride;
    t.results.assign(static_cast<size_t>(stride) * t.scores.size() * 3, 0.0);
  }

  // coordinate depth
  std::function<int(int, int)> depth = [&](int u, int d) -> int {
    if (d > 8) throw std::runtime_error("universe nesting is too deep or cyclic");
    int best = 1;
    for (int c : m.universes[u]) {
      const HCell& cell = m.cells[c];
      if (cell.fill_type == FILL_UNIVERSE) best = std::max(best, 1 + depth(cell.fill, d + 1));
      if (cell.fill_type == FILL_LATTICE) {
        const HLattice& lat = m.lattices[cell.fill];
        std::vector<int> seen;
        for (int lu : lat.univ) {
          if (std::find(seen.begin(), seen.end(), lu) != seen.end()) continue;
          seen.push_back(lu);
          best = std::max(best, 1 + depth(lu, d + 1));
        }
        if (lat.outer >= 0) best = std::max(best, 1 + depth(lat.outer, d + 1));
      }
    }
    return best;
  };
  m.n_coord_levels = depth(m.root_universe, 0);
}

}  // namespace omc
