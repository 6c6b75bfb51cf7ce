// Checker of openmc_gb300/csrc/h5lite.cpp against the Python reader
// (openmc_gb300/h5.py), driven by tests/test_h5.py.
//
//   h5lite_check dump <file>    prints every group, dataset and attribute of
//                               the file, one line each, in a canonical form
//   h5lite_check write <file>   writes a tree holding every value kind the
//                               writer supports
//
// Dump lines: "<path> G" for a group, "<path> D <value>" for a dataset,
// "<path>@<name> A <value>" for an attribute.  A value is its kind, its
// shape, and its elements (strings as text, numbers with %.17g).
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../openmc_gb300/csrc/h5lite.h"

using namespace omc;

namespace {

std::string show(const h5::Value& v)
{
  std::string out(1, v.kind);
  out += " (";
  for (size_t k = 0; k < v.shape.size(); ++k) out += (k ? "," : "") + std::to_string(v.shape[k]);
  out += ")";
  char buf[64];
  if (v.kind == 's') {
    const size_t n = v.count();
    for (size_t k = 0; k < n; ++k) {
      std::string e(reinterpret_cast<const char*>(v.bytes.data()) + k * v.size, v.size);
      e = e.substr(0, e.find('\0'));
      out += " '" + e + "'";
    }
  } else if (v.kind == 'f') {
    for (double d : v.doubles()) {
      std::snprintf(buf, sizeof(buf), " %.17g", d);
      out += buf;
    }
  } else if (v.kind == 'u') {
    for (size_t k = 0; k < v.count(); ++k) {
      unsigned long long x = 0;
      for (size_t j = 0; j < v.size; ++j) x |= static_cast<unsigned long long>(v.bytes[k * v.size + j]) << (8 * j);
      out += " " + std::to_string(x);
    }
  } else {
    for (long long i : v.ints()) out += " " + std::to_string(i);
  }
  return out;
}

// depth-limited: a corrupt file can make a group its own descendant
void dump(const h5::Node& n, const std::string& path, int depth = 0)
{
  if (depth > 32) throw std::runtime_error("groups nested too deeply (a cycle?)");
  for (const auto& a : n.attr_names()) std::printf("%s@%s A %s\n", path.c_str(), a.c_str(), show(n.attr(a)).c_str());
  if (n.is_dataset()) {
    std::printf("%s D %s\n", path.c_str(), show(n.read()).c_str());
    return;
  }
  std::printf("%s G\n", path.c_str());
  for (const auto& c : n.children()) dump(n.at(c), path + "/" + c, depth + 1);
}

}  // namespace

int main(int argc, char** argv)
{
  if (argc != 3) {
    std::fprintf(stderr, "usage: h5lite_check dump|write <file>\n");
    return 2;
  }
  try {
    const std::string mode = argv[1];
    if (mode == "dump") {
      h5::File f(argv[2]);
      dump(f.root(), "");
      return 0;
    }
    if (mode == "write") {
      h5::WNode root;
      root.attrs["filetype"] = h5::string("check");
      root.attrs["version"] = h5::array(std::vector<long long> {18, 1});
      root.attrs["scale"] = h5::scalar(0.1);
      root.dataset("n", h5::scalar(42LL));
      root.dataset("x", h5::scalar(-2.5e-300));
      root.dataset("name", h5::string("a name"));
      std::vector<double> grid;
      for (int k = 0; k < 3 * 4 * 2; ++k) grid.push_back(1.0 / (k + 1));
      root.dataset("grid", h5::array(grid, {3, 4, 2})).attrs["units"] = h5::string("cm");
      h5::WNode& g = root.group_at("tallies");
      g.attrs["n"] = h5::scalar(150LL);
      // more members than one symbol-table node holds
      for (int k = 0; k < 150; ++k) {
        h5::WNode& t = g.group_at("tally " + std::to_string(k + 1));
        t.dataset("results", h5::array(std::vector<double> {double(k), double(k) * k}, {1, 1, 2}));
        t.attrs["id"] = h5::scalar(static_cast<long long>(k + 1));
      }
      root.group_at("empty");
      h5::write(argv[2], root);
      return 0;
    }
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
}
