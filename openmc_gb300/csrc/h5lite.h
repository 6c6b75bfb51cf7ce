// A small HDF5 reader and writer for the files this library exchanges with
// the reference's tools: incident-neutron nuclide files (read at
// openmc_init, docs/source/io_formats/nuclear_data.rst) and statepoints
// (written by openmc_statepoint_write, docs/source/io_formats/statepoint.rst).
// libhdf5 is not available, so the subset of the HDF5 file format these files
// use is implemented from the format specification:
//   - superblock version 0 (written) and 0/1/2/3 (read), 8-byte offsets;
//   - groups in the "symbol table" form (version-1 B-tree, symbol-table
//     nodes, local heap), as h5py writes by default, and compact link
//     messages (read);
//   - object headers version 1 (written) and 1/2 (read) with continuations;
//   - contiguous and compact datasets (no chunking, no filters);
//   - little-endian IEEE floats, integers and fixed-length strings
//     (enumerations read as their base integers).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace omc {
namespace h5 {

struct Value {
  char kind = 0;  // 'f' float, 'i' signed, 'u' unsigned, 's' string
  size_t size = 0;  // bytes per element
  std::vector<uint64_t> shape;  // empty: scalar
  std::vector<uint8_t> bytes;
  size_t count() const;
  std::vector<double> doubles() const;
  std::vector<long long> ints() const;
  std::string str() const;  // first string element, without trailing NULs
};

class File;

// A group or dataset of a file being read.
class Node {
 public:
  Node(const File* f, uint64_t addr) : f_(f), addr_(addr) {}
  bool is_dataset() const;
  bool has(const std::string& path) const;
  Node at(const std::string& path) const;  // "a/b/c" below this group
  std::vector<std::string> children() const;  // member names in name order
  bool has_attr(const std::string& name) const;
  Value attr(const std::string& name) const;
  std::vector<std::string> attr_names() const;  // in header order
  Value read() const;  // the dataset's value
 private:
  const File* f_;
  uint64_t addr_;
};

class File {
 public:
  explicit File(const std::string& path);
  Node root() const;
  // internal
  struct Msg {
    int type;
    uint64_t pos, size;
  };
  std::vector<Msg> messages(uint64_t addr) const;
  std::vector<std::pair<std::string, uint64_t>> members(uint64_t addr) const;
  Value datatype_value(uint64_t p) const;  // kind and size only
  std::vector<uint64_t> dataspace(uint64_t p) const;
  uint64_t u(uint64_t off, int n) const;  // little-endian n-byte integer (bounds-checked)
  bool tag(uint64_t off, const char* t) const;
  std::string bytes_at(uint64_t off, uint64_t len) const;
  std::string cstr_at(uint64_t off) const;
  const std::vector<uint8_t>& bytes() const { return b_; }
  const std::string& path() const { return path_; }
 private:
  std::string path_;
  std::vector<uint8_t> b_;
  uint64_t root_ = 0;
};

// ------------------------------------------------------------------ writing
// A tree to write: groups hold named children and attributes; datasets
// hold a value and attributes.
struct WNode {
  bool group = true;
  Value value;
  std::map<std::string, Value> attrs;
  std::map<std::string, std::shared_ptr<WNode>> children;
  WNode& group_at(const std::string& name);  // creates a sub-group
  WNode& dataset(const std::string& name, Value v);
};

Value scalar(double v);
Value scalar(long long v);
Value string(const std::string& s);
Value array(const std::vector<double>& v, std::vector<uint64_t> shape = {});
Value array(const std::vector<long long>& v, std::vector<uint64_t> shape = {});

void write(const std::string& path, const WNode& root);

}  // namespace h5
}  // namespace omc
