// HDF5 subset reader and writer (see h5lite.h).  Structures follow the HDF5
// file format specification, version 2 and later: superblock, version-1
// B-trees of group nodes, symbol-table nodes, local heaps, object headers
// (versions 1 and 2) and the dataspace, datatype, layout, attribute,
// link, symbol-table and continuation messages.
#include "h5lite.h"

#include <algorithm>
#include <array>
#include <cstring>
#include <fstream>
#include <stdexcept>

namespace omc {
namespace h5 {

namespace {

constexpr uint64_t UNDEF = ~0ull;
const uint8_t SIGNATURE[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

enum {
  MSG_NIL = 0, MSG_DATASPACE = 1, MSG_LINK_INFO = 2, MSG_DATATYPE = 3, MSG_FILL = 5, MSG_LINK = 6,
  MSG_LAYOUT = 8, MSG_ATTRIBUTE = 12, MSG_CONTINUATION = 16, MSG_SYMBOL_TABLE = 17
};

[[noreturn]] void fail(const File& f, const std::string& what)
{
  throw std::runtime_error(f.path() + ": " + what);
}

uint64_t pad8(uint64_t n) { return (n + 7) & ~7ull; }

std::vector<std::string> split_path(const std::string& p)
{
  std::vector<std::string> out;
  size_t a = 0;
  while (a < p.size()) {
    size_t b = p.find('/', a);
    if (b == std::string::npos) b = p.size();
    if (b > a) out.push_back(p.substr(a, b - a));
    a = b + 1;
  }
  return out;
}

}  // namespace

// ------------------------------------------------------------------ values
size_t Value::count() const
{
  size_t n = 1;
  for (uint64_t d : shape) {
    if (d != 0 && n > (uint64_t(1) << 40) / d) throw std::runtime_error("HDF5 dataspace too large");
    n *= d;
  }
  return n;
}

std::vector<double> Value::doubles() const
{
  const size_t n = count();
  std::vector<double> out(n);
  for (size_t k = 0; k < n; ++k) {
    const uint8_t* p = bytes.data() + k * size;
    if (kind == 'f' && size == 8) {
      std::memcpy(&out[k], p, 8);
    } else if (kind == 'f' && size == 4) {
      float f;
      std::memcpy(&f, p, 4);
      out[k] = f;
    } else if (kind == 'i' || kind == 'u') {
      uint64_t v = 0;
      std::memcpy(&v, p, size);
      if (kind == 'i' && size < 8 && (v >> (8 * size - 1)) & 1) v |= ~0ull << (8 * size);
      out[k] = kind == 'i' ? static_cast<double>(static_cast<long long>(v)) : static_cast<double>(v);
    } else {
      throw std::runtime_error("HDF5 value is not numeric");
    }
  }
  return out;
}

std::vector<long long> Value::ints() const
{
  const size_t n = count();
  std::vector<long long> out(n);
  if (kind == 'f') {
    const std::vector<double> d = doubles();
    for (size_t k = 0; k < n; ++k) out[k] = static_cast<long long>(d[k]);
    return out;
  }
  for (size_t k = 0; k < n; ++k) {
    const uint8_t* p = bytes.data() + k * size;
    if (kind == 'i' || kind == 'u') {
      uint64_t v = 0;
      std::memcpy(&v, p, size);
      if (kind == 'i' && size < 8 && (v >> (8 * size - 1)) & 1) v |= ~0ull << (8 * size);
      out[k] = static_cast<long long>(v);
    } else {
      throw std::runtime_error("HDF5 value is not numeric");
    }
  }
  return out;
}

std::string Value::str() const
{
  if (kind != 's') throw std::runtime_error("HDF5 value is not a string");
  std::string s(reinterpret_cast<const char*>(bytes.data()), std::min(size, bytes.size()));
  while (!s.empty() && (s.back() == '\0' || s.back() == ' ')) s.pop_back();
  return s;
}

// ------------------------------------------------------------------ reading
File::File(const std::string& path) : path_(path)
{
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("cannot open " + path);
  b_.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
  if (b_.size() < 96 || std::memcmp(b_.data(), SIGNATURE, 8) != 0) fail(*this, "not an HDF5 file");
  const int ver = b_[8];
  if (ver == 0 || ver == 1) {
    if (b_[13] != 8 || b_[14] != 8) fail(*this, "only 8-byte offsets and lengths are supported");
    const uint64_t entry = 24 + (ver == 1 ? 4 : 0) + 32;
    root_ = u(entry + 8, 8);
  } else if (ver == 2 || ver == 3) {
    if (b_[9] != 8 || b_[10] != 8) fail(*this, "only 8-byte offsets and lengths are supported");
    root_ = u(12 + 24, 8);
  } else {
    fail(*this, "unsupported superblock version");
  }
}

uint64_t File::u(uint64_t off, int n) const
{
  if (off > b_.size() || static_cast<uint64_t>(n) > b_.size() - off) fail(*this, "read past the end of the file");
  uint64_t v = 0;
  for (int k = n - 1; k >= 0; --k) v = (v << 8) | b_[off + k];
  return v;
}

// Whether the 4-byte signature t stands at off (false past the end).
bool File::tag(uint64_t off, const char* t) const
{
  return off <= b_.size() && b_.size() - off >= 4 && std::memcmp(&b_[off], t, 4) == 0;
}

// len bytes at off as a string (failing past the end of the file).
std::string File::bytes_at(uint64_t off, uint64_t len) const
{
  if (off > b_.size() || len > b_.size() - off) fail(*this, "read past the end of the file");
  return std::string(reinterpret_cast<const char*>(&b_[off]), len);
}

// The NUL-terminated string at off (failing when it runs past the end).
std::string File::cstr_at(uint64_t off) const
{
  if (off >= b_.size()) fail(*this, "read past the end of the file");
  const void* end = std::memchr(&b_[off], 0, b_.size() - off);
  if (!end) fail(*this, "unterminated string");
  return std::string(reinterpret_cast<const char*>(&b_[off]), static_cast<const uint8_t*>(end) - &b_[off]);
}

Node File::root() const { return Node(this, root_); }

std::vector<File::Msg> File::messages(uint64_t addr) const
{
  std::vector<Msg> out;
  if (tag(addr, "OHDR")) {
    const int flags = static_cast<int>(u(addr + 5, 1));
    uint64_t off = addr + 6;
    if (flags & 0x20) off += 16;
    if (flags & 0x10) off += 4;
    const int size_len = 1 << (flags & 3);
    const uint64_t chunk = u(off, size_len);
    off += size_len;
    std::vector<std::pair<uint64_t, uint64_t>> blocks {{off, chunk}};
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      if (bi >= 4096) fail(*this, "too many object header continuations");
      uint64_t p = blocks[bi].first, end = blocks[bi].first + blocks[bi].second;
      while (p + 4 <= end) {
        const int type = static_cast<int>(u(p, 1));
        const uint64_t size = u(p + 1, 2);
        p += 4 + ((flags & 0x04) ? 2 : 0);
        if (type == MSG_CONTINUATION) {
          const uint64_t ca = u(p, 8), cl = u(p + 8, 8);
          if (!tag(ca, "OCHK") || cl < 8) fail(*this, "bad object header continuation");
          blocks.push_back({ca + 4, cl - 8});
        } else {
          out.push_back({type, p, size});
        }
        p += size;
      }
    }
    return out;
  }
  if (u(addr, 1) != 1) fail(*this, "unsupported object header version");
  const uint64_t nmsg = u(addr + 2, 2), hsize = u(addr + 8, 4);
  std::vector<std::pair<uint64_t, uint64_t>> blocks {{addr + 16, hsize}};
  uint64_t count = 0;
  for (size_t bi = 0; bi < blocks.size() && count < nmsg; ++bi) {
    if (bi >= 4096) fail(*this, "too many object header continuations");
    uint64_t p = blocks[bi].first, end = blocks[bi].first + blocks[bi].second;
    while (p + 8 <= end && count < nmsg) {
      const int type = static_cast<int>(u(p, 2));
      const uint64_t size = u(p + 2, 2);
      p += 8;
      ++count;
      if (type == MSG_CONTINUATION) blocks.push_back({u(p, 8), u(p + 8, 8)});
      else out.push_back({type, p, size});
      p += size;
    }
  }
  return out;
}

Value File::datatype_value(uint64_t p) const
{
  Value v;
  const int cls = static_cast<int>(u(p, 1)) & 0x0F;
  const int bits0 = static_cast<int>(u(p + 1, 1));
  v.size = u(p + 4, 4);
  if (cls == 0) {
    if (bits0 & 1) fail(*this, "big-endian integers are not supported");
    if (v.size != 1 && v.size != 2 && v.size != 4 && v.size != 8) fail(*this, "unsupported integer size");
    v.kind = (bits0 & 0x08) ? 'i' : 'u';
  } else if (cls == 1) {
    if ((bits0 & 1) || (v.size != 4 && v.size != 8)) fail(*this, "only little-endian IEEE floats are supported");
    v.kind = 'f';
  } else if (cls == 3) {
    if (v.size == 0) fail(*this, "empty string type");
    v.kind = 's';
  } else if (cls == 8) {
    // enumeration: its base type (one level; a nested enumeration is not
    // what h5py writes)
    if ((u(p + 8, 1) & 0x0F) == 8) fail(*this, "nested enumeration types are not supported");
    return datatype_value(p + 8);
  } else {
    fail(*this, "unsupported datatype class " + std::to_string(cls));
  }
  return v;
}

std::vector<uint64_t> File::dataspace(uint64_t p) const
{
  const int ver = static_cast<int>(u(p, 1)), ndim = static_cast<int>(u(p + 1, 1));
  uint64_t q;
  if (ver == 1) q = p + 8;
  else if (ver == 2) q = p + 4;
  else fail(*this, "unsupported dataspace version");
  std::vector<uint64_t> dims(ndim);
  for (int k = 0; k < ndim; ++k) dims[k] = u(q + 8 * k, 8);
  return dims;
}

std::vector<std::pair<std::string, uint64_t>> File::members(uint64_t addr) const
{
  std::vector<std::pair<std::string, uint64_t>> out;
  for (const Msg& m : messages(addr)) {
    if (m.type == MSG_SYMBOL_TABLE) {
      const uint64_t btree = u(m.pos, 8), heap = u(m.pos + 8, 8);
      if (!tag(heap, "HEAP")) fail(*this, "bad local heap");
      const uint64_t data = u(heap + 24, 8);
      std::vector<uint64_t> stack {btree};
      size_t visited = 0;
      while (!stack.empty()) {
        if (++visited > (1u << 20)) fail(*this, "B-tree too large or cyclic");
        const uint64_t node = stack.back();
        stack.pop_back();
        if (!tag(node, "TREE")) fail(*this, "bad B-tree node");
        const int level = static_cast<int>(u(node + 5, 1));
        const uint64_t used = u(node + 6, 2);
        std::vector<uint64_t> kids;
        for (uint64_t k = 0; k < used; ++k) kids.push_back(u(node + 24 + 8 + 16 * k, 8));
        if (level > 0) {
          for (auto it = kids.rbegin(); it != kids.rend(); ++it) stack.push_back(*it);
          continue;
        }
        for (uint64_t sn : kids) {
          if (!tag(sn, "SNOD")) fail(*this, "bad symbol table node");
          const uint64_t n = u(sn + 6, 2);
          for (uint64_t k = 0; k < n; ++k) {
            const uint64_t e = sn + 8 + 40 * k;
            out.push_back({cstr_at(data + u(e, 8)), u(e + 8, 8)});
          }
        }
      }
    } else if (m.type == MSG_LINK) {
      const int flags = static_cast<int>(u(m.pos + 1, 1));
      uint64_t q = m.pos + 2;
      int ltype = 0;
      if (flags & 0x08) ltype = static_cast<int>(u(q++, 1));
      if (flags & 0x04) q += 8;
      if (flags & 0x10) q += 1;
      const int nl = 1 << (flags & 3);
      const uint64_t len = u(q, nl);
      q += nl;
      std::string name = bytes_at(q, len);
      q += len;
      if (ltype == 0) out.push_back({name, u(q, 8)});
    } else if (m.type == MSG_LINK_INFO) {
      const uint64_t fh = u(m.pos + 2 + ((u(m.pos + 1, 1) & 1) ? 8 : 0), 8);
      if (fh != UNDEF) fail(*this, "groups with dense link storage are not supported");
    }
  }
  std::sort(out.begin(), out.end());
  return out;
}

bool Node::is_dataset() const
{
  for (const auto& m : f_->messages(addr_))
    if (m.type == MSG_LAYOUT) return true;
  return false;
}

bool Node::has(const std::string& path) const
{
  uint64_t a = addr_;
  for (const std::string& part : split_path(path)) {
    bool found = false;
    for (const auto& kv : f_->members(a))
      if (kv.first == part) {
        a = kv.second;
        found = true;
        break;
      }
    if (!found) return false;
  }
  return true;
}

Node Node::at(const std::string& path) const
{
  uint64_t a = addr_;
  for (const std::string& part : split_path(path)) {
    bool found = false;
    for (const auto& kv : f_->members(a))
      if (kv.first == part) {
        a = kv.second;
        found = true;
        break;
      }
    if (!found) throw std::runtime_error(f_->path() + ": no object '" + path + "'");
  }
  return Node(f_, a);
}

std::vector<std::string> Node::children() const
{
  std::vector<std::string> out;
  for (const auto& kv : f_->members(addr_)) out.push_back(kv.first);
  return out;
}

namespace {

// attribute message -> (name, value)
std::pair<std::string, Value> parse_attribute(const File& f, uint64_t p)
{
  const auto& b = f.bytes();
  const int ver = static_cast<int>(f.u(p, 1));
  const uint64_t name_size = f.u(p + 2, 2), dt_size = f.u(p + 4, 2), ds_size = f.u(p + 6, 2);
  uint64_t q;
  std::string name;
  Value v;
  if (ver == 1) {
    q = p + 8;
    name = f.cstr_at(q);
    q += pad8(name_size);
    v = f.datatype_value(q);
    q += pad8(dt_size);
    v.shape = f.dataspace(q);
    q += pad8(ds_size);
  } else if (ver == 2 || ver == 3) {
    q = p + 8 + (ver == 3 ? 1 : 0);
    name = f.cstr_at(q);
    q += name_size;
    v = f.datatype_value(q);
    q += dt_size;
    v.shape = f.dataspace(q);
    q += ds_size;
  } else {
    throw std::runtime_error(f.path() + ": unsupported attribute version");
  }
  const size_t n = v.count() * v.size;
  if (q > b.size() || n > b.size() - q) throw std::runtime_error(f.path() + ": attribute past the end of the file");
  v.bytes.assign(b.begin() + q, b.begin() + q + n);
  return {name, v};
}

}  // namespace

bool Node::has_attr(const std::string& name) const
{
  for (const auto& m : f_->messages(addr_))
    if (m.type == MSG_ATTRIBUTE && parse_attribute(*f_, m.pos).first == name) return true;
  return false;
}

std::vector<std::string> Node::attr_names() const
{
  std::vector<std::string> out;
  for (const auto& m : f_->messages(addr_))
    if (m.type == MSG_ATTRIBUTE) out.push_back(parse_attribute(*f_, m.pos).first);
  return out;
}

Value Node::attr(const std::string& name) const
{
  for (const auto& m : f_->messages(addr_))
    if (m.type == MSG_ATTRIBUTE) {
      auto kv = parse_attribute(*f_, m.pos);
      if (kv.first == name) return kv.second;
    }
  throw std::runtime_error(f_->path() + ": no attribute '" + name + "'");
}

Value Node::read() const
{
  Value v;
  bool have_type = false, have_space = false, have_layout = false;
  uint64_t addr = UNDEF, size = 0;
  uint64_t compact = UNDEF;  // file offset of a compact dataset's bytes
  for (const auto& m : f_->messages(addr_)) {
    if (m.type == MSG_DATATYPE) {
      const Value t = f_->datatype_value(m.pos);
      v.kind = t.kind;
      v.size = t.size;
      have_type = true;
    } else if (m.type == MSG_DATASPACE) {
      v.shape = f_->dataspace(m.pos);
      have_space = true;
    } else if (m.type == MSG_LAYOUT) {
      if (f_->u(m.pos, 1) != 3) throw std::runtime_error(f_->path() + ": unsupported data layout version");
      const int cls = static_cast<int>(f_->u(m.pos + 1, 1));
      if (cls == 0) {
        size = f_->u(m.pos + 2, 2);
        compact = m.pos + 4;
      } else if (cls == 1) {
        addr = f_->u(m.pos + 2, 8);
        size = f_->u(m.pos + 10, 8);
      } else {
        throw std::runtime_error(f_->path() + ": chunked datasets are not supported");
      }
      have_layout = true;
    }
  }
  if (!have_type || !have_space || !have_layout) throw std::runtime_error(f_->path() + ": not a dataset");
  const size_t n = v.count() * v.size;
  if (n > (uint64_t(1) << 36)) throw std::runtime_error(f_->path() + ": dataset too large");
  if (compact != UNDEF) {
    const std::string c = f_->bytes_at(compact, std::min<uint64_t>(n, size));
    v.bytes.assign(c.begin(), c.end());
  } else if (addr == UNDEF) {
    v.bytes.assign(n, 0);
  } else {
    const auto& b = f_->bytes();
    if (addr > b.size() || n > b.size() - addr) throw std::runtime_error(f_->path() + ": dataset past the end of the file");
    v.bytes.assign(b.begin() + addr, b.begin() + addr + n);
  }
  v.bytes.resize(n, 0);
  return v;
}

// ------------------------------------------------------------------ writing
WNode& WNode::group_at(const std::string& name)
{
  auto& c = children[name];
  if (!c) c = std::make_shared<WNode>();
  return *c;
}

WNode& WNode::dataset(const std::string& name, Value v)
{
  auto& c = children[name];
  c = std::make_shared<WNode>();
  c->group = false;
  c->value = std::move(v);
  return *c;
}

Value scalar(double x)
{
  Value v;
  v.kind = 'f';
  v.size = 8;
  v.bytes.resize(8);
  std::memcpy(v.bytes.data(), &x, 8);
  return v;
}

Value scalar(long long x)
{
  Value v;
  v.kind = 'i';
  v.size = 8;
  v.bytes.resize(8);
  std::memcpy(v.bytes.data(), &x, 8);
  return v;
}

Value string(const std::string& s)
{
  Value v;
  v.kind = 's';
  v.size = std::max<size_t>(s.size(), 1);
  v.bytes.assign(s.begin(), s.end());
  v.bytes.resize(v.size, 0);
  return v;
}

Value array(const std::vector<double>& a, std::vector<uint64_t> shape)
{
  Value v;
  v.kind = 'f';
  v.size = 8;
  v.shape = shape.empty() ? std::vector<uint64_t> {a.size()} : shape;
  v.bytes.resize(a.size() * 8);
  if (!a.empty()) std::memcpy(v.bytes.data(), a.data(), a.size() * 8);
  return v;
}

Value array(const std::vector<long long>& a, std::vector<uint64_t> shape)
{
  Value v;
  v.kind = 'i';
  v.size = 8;
  v.shape = shape.empty() ? std::vector<uint64_t> {a.size()} : shape;
  v.bytes.resize(a.size() * 8);
  if (!a.empty()) std::memcpy(v.bytes.data(), a.data(), a.size() * 8);
  return v;
}

namespace {

struct Out {
  std::vector<uint8_t> b;
  static constexpr int LEAF_K = 64, INTERNAL_K = 16;
  Out() : b(96, 0) {}
  void put(std::vector<uint8_t>& v, uint64_t x, int n)
  {
    for (int k = 0; k < n; ++k) v.push_back(static_cast<uint8_t>(x >> (8 * k)));
  }
  uint64_t alloc(const std::vector<uint8_t>& data)
  {
    const uint64_t a = b.size();
    b.insert(b.end(), data.begin(), data.end());
    b.resize(pad8(b.size()), 0);
    return a;
  }
  std::vector<uint8_t> datatype(const Value& v)
  {
    std::vector<uint8_t> m;
    if (v.kind == 'f') {
      m = {0x11, 0x20, static_cast<uint8_t>(v.size * 8 - 1), 0};
      put(m, v.size, 4);
      if (v.size == 8) {
        put(m, 0, 2); put(m, 64, 2); m.push_back(52); m.push_back(11); m.push_back(0); m.push_back(52);
        put(m, 1023, 4);
      } else {
        put(m, 0, 2); put(m, 32, 2); m.push_back(23); m.push_back(8); m.push_back(0); m.push_back(23);
        put(m, 127, 4);
      }
    } else if (v.kind == 'i' || v.kind == 'u') {
      m = {0x10, static_cast<uint8_t>(v.kind == 'i' ? 0x08 : 0), 0, 0};
      put(m, v.size, 4);
      put(m, 0, 2);
      put(m, v.size * 8, 2);
    } else {
      m = {0x13, 0x00, 0, 0};  // null-terminated ASCII string
      put(m, v.size, 4);
    }
    return m;
  }
  std::vector<uint8_t> dataspace(const Value& v)
  {
    std::vector<uint8_t> m = {1, static_cast<uint8_t>(v.shape.size()), 0, 0, 0, 0, 0, 0};
    for (uint64_t d : v.shape) put(m, d, 8);
    return m;
  }
  static void pad(std::vector<uint8_t>& v) { v.resize(pad8(v.size()), 0); }
  std::vector<uint8_t> attribute(const std::string& name, const Value& v)
  {
    std::vector<uint8_t> nm(name.begin(), name.end());
    nm.push_back(0);
    auto dt = datatype(v), ds = dataspace(v);
    std::vector<uint8_t> m = {1, 0};
    put(m, nm.size(), 2);
    put(m, dt.size(), 2);
    put(m, ds.size(), 2);
    pad(nm); pad(dt); pad(ds);
    m.insert(m.end(), nm.begin(), nm.end());
    m.insert(m.end(), dt.begin(), dt.end());
    m.insert(m.end(), ds.begin(), ds.end());
    m.insert(m.end(), v.bytes.begin(), v.bytes.end());
    return m;
  }
  uint64_t header(std::vector<std::pair<int, std::vector<uint8_t>>> msgs)
  {
    std::vector<uint8_t> body;
    if (msgs.empty()) msgs.push_back({MSG_NIL, std::vector<uint8_t>(8, 0)});
    for (auto& [type, payload] : msgs) {
      pad(payload);
      put(body, type, 2);
      put(body, payload.size(), 2);
      body.insert(body.end(), {0, 0, 0, 0});
      body.insert(body.end(), payload.begin(), payload.end());
    }
    std::vector<uint8_t> h = {1, 0};
    put(h, msgs.size(), 2);
    put(h, 1, 4);
    put(h, body.size(), 4);
    put(h, 0, 4);
    h.insert(h.end(), body.begin(), body.end());
    return alloc(h);
  }
  std::vector<std::pair<int, std::vector<uint8_t>>> attr_msgs(const WNode& n)
  {
    std::vector<std::pair<int, std::vector<uint8_t>>> out;
    for (const auto& [k, v] : n.attrs) out.push_back({MSG_ATTRIBUTE, attribute(k, v)});
    return out;
  }
  uint64_t dataset(const WNode& n)
  {
    const Value& v = n.value;
    const uint64_t addr = v.bytes.empty() ? UNDEF : alloc(v.bytes);
    std::vector<uint8_t> layout = {3, 1};
    put(layout, addr, 8);
    put(layout, v.bytes.size(), 8);
    std::vector<std::pair<int, std::vector<uint8_t>>> msgs = {
      {MSG_DATASPACE, dataspace(v)}, {MSG_DATATYPE, datatype(v)}, {MSG_FILL, {2, 2, 2, 0}}, {MSG_LAYOUT, layout}};
    for (auto& m : attr_msgs(n)) msgs.push_back(m);
    return header(msgs);
  }
  // returns (object header, B-tree, heap)
  std::array<uint64_t, 3> group(const WNode& n)
  {
    // one B-tree leaf node over up to 2 INTERNAL_K symbol-table nodes of up
    // to 2 LEAF_K entries each; key k + 1 is the last name of node k
    if (n.children.size() > size_t(2 * LEAF_K) * 2 * INTERNAL_K)
      throw std::runtime_error("HDF5 groups of more than 4096 members are not supported");
    std::vector<std::string> names;
    std::vector<uint64_t> kids;
    for (const auto& [name, c] : n.children) {  // std::map: name order
      names.push_back(name);
      kids.push_back(c->group ? group(*c)[0] : dataset(*c));
    }
    std::vector<uint8_t> heap_data(8, 0);
    std::vector<uint64_t> offs;
    for (const auto& name : names) {
      offs.push_back(heap_data.size());
      heap_data.insert(heap_data.end(), name.begin(), name.end());
      heap_data.push_back(0);
      pad(heap_data);
    }
    heap_data.resize(heap_data.size() + 8, 0);
    const uint64_t data_addr = alloc(heap_data);
    std::vector<uint8_t> heap = {'H', 'E', 'A', 'P', 0, 0, 0, 0};
    put(heap, heap_data.size(), 8);
    put(heap, UNDEF, 8);
    put(heap, data_addr, 8);
    const uint64_t heap_addr = alloc(heap);
    std::vector<uint64_t> snods, last;
    for (size_t k0 = 0; k0 == 0 || k0 < names.size(); k0 += 2 * LEAF_K) {
      const size_t k1 = std::min(names.size(), k0 + 2 * LEAF_K);
      std::vector<uint8_t> snod = {'S', 'N', 'O', 'D', 1, 0};
      put(snod, k1 - k0, 2);
      for (size_t k = k0; k < k1; ++k) {
        put(snod, offs[k], 8);
        put(snod, kids[k], 8);
        put(snod, 0, 8);
        snod.resize(snod.size() + 16, 0);
      }
      snod.resize(8 + 40 * 2 * LEAF_K, 0);
      snods.push_back(alloc(snod));
      last.push_back(k1 > k0 ? offs[k1 - 1] : 0);
    }
    std::vector<uint8_t> tree = {'T', 'R', 'E', 'E', 0, 0};
    put(tree, snods.size(), 2);
    put(tree, UNDEF, 8);
    put(tree, UNDEF, 8);
    put(tree, 0, 8);
    for (size_t k = 0; k < snods.size(); ++k) {
      put(tree, snods[k], 8);
      put(tree, last[k], 8);
    }
    tree.resize(24 + 8 + 16 * 2 * INTERNAL_K, 0);
    const uint64_t tree_addr = alloc(tree);
    std::vector<uint8_t> stab;
    put(stab, tree_addr, 8);
    put(stab, heap_addr, 8);
    std::vector<std::pair<int, std::vector<uint8_t>>> msgs = {{MSG_SYMBOL_TABLE, stab}};
    for (auto& m : attr_msgs(n)) msgs.push_back(m);
    return {header(msgs), tree_addr, heap_addr};
  }
};

}  // namespace

void write(const std::string& path, const WNode& root)
{
  Out o;
  const auto r = o.group(root);
  std::vector<uint8_t> sb(SIGNATURE, SIGNATURE + 8);
  sb.insert(sb.end(), {0, 0, 0, 0, 0, 8, 8, 0});
  o.put(sb, Out::LEAF_K, 2);
  o.put(sb, Out::INTERNAL_K, 2);
  o.put(sb, 0, 4);
  o.put(sb, 0, 8);
  o.put(sb, UNDEF, 8);
  o.put(sb, o.b.size(), 8);
  o.put(sb, UNDEF, 8);
  o.put(sb, 0, 8);
  o.put(sb, r[0], 8);
  o.put(sb, 1, 4);
  o.put(sb, 0, 4);
  o.put(sb, r[1], 8);
  o.put(sb, r[2], 8);
  std::copy(sb.begin(), sb.end(), o.b.begin());
  std::ofstream out(path, std::ios::binary);
  if (!out) throw std::runtime_error("cannot write " + path);
  out.write(reinterpret_cast<const char*>(o.b.data()), static_cast<std::streamsize>(o.b.size()));
  if (!out) throw std::runtime_error("error writing " + path);
}

}  // namespace h5
}  // namespace omc
