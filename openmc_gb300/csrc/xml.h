// Minimal XML DOM reader for OpenMC input files.
//
// OpenMC reads model.xml / settings.xml / geometry.xml / materials.xml /
// tallies.xml / cross_sections.xml with pugixml (src/xml_interface.cpp).  This
// reader covers what those files use: a prolog, comments, elements with
// attributes, text content, self-closing tags, CDATA and the five predefined
// entities.  Lookups mirror the reference helpers: check_for_node() accepts an
// attribute or a child element, get_node_value() returns either one's text.
#pragma once

#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace omc {

struct XmlNode {
  std::string name;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::string text;
  std::vector<std::unique_ptr<XmlNode>> children;

  const std::string* attr(const std::string& k) const
  {
    for (const auto& a : attrs)
      if (a.first == k) return &a.second;
    return nullptr;
  }
  const XmlNode* child(const std::string& k) const
  {
    for (const auto& c : children)
      if (c->name == k) return c.get();
    return nullptr;
  }
  std::vector<const XmlNode*> all(const std::string& k) const
  {
    std::vector<const XmlNode*> out;
    for (const auto& c : children)
      if (c->name == k) out.push_back(c.get());
    return out;
  }
  // Attribute or child-element text (src/xml_interface.cpp get_node_value)
  bool has(const std::string& k) const { return attr(k) || child(k); }
  std::string value(const std::string& k) const
  {
    if (auto a = attr(k)) return trim(*a);
    if (auto c = child(k)) return trim(c->text);
    throw std::runtime_error("missing <" + k + "> in <" + name + ">");
  }
  std::string value_or(const std::string& k, const std::string& d) const { return has(k) ? value(k) : d; }

  static std::string trim(const std::string& s)
  {
    size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
  }
};

inline std::vector<double> split_doubles(const std::string& s)
{
  std::vector<double> out;
  const char* p = s.c_str();
  char* end;
  while (*p) {
    while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') ++p;
    if (!*p) break;
    double v = std::strtod(p, &end);
    if (end == p) throw std::runtime_error("bad number in '" + s.substr(0, 40) + "'");
    out.push_back(v);
    p = end;
  }
  return out;
}

inline std::vector<long long> split_ints(const std::string& s)
{
  std::vector<long long> out;
  const char* p = s.c_str();
  char* end;
  while (*p) {
    while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') ++p;
    if (!*p) break;
    long long v = std::strtoll(p, &end, 10);
    if (end == p) throw std::runtime_error("bad integer in '" + s.substr(0, 40) + "'");
    out.push_back(v);
    p = end;
  }
  return out;
}

inline std::vector<std::string> split_words(const std::string& s)
{
  std::vector<std::string> out;
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && isspace(static_cast<unsigned char>(s[i]))) ++i;
    size_t j = i;
    while (j < s.size() && !isspace(static_cast<unsigned char>(s[j]))) ++j;
    if (j > i) out.push_back(s.substr(i, j - i));
    i = j;
  }
  return out;
}

class XmlParser {
public:
  explicit XmlParser(const std::string& src) : s_(src) {}

  std::unique_ptr<XmlNode> parse()
  {
    skip_misc();
    if (!peek('<')) throw err("expected root element");
    auto root = element();
    return root;
  }

private:
  const std::string& s_;
  size_t i_ = 0;

  std::runtime_error err(const std::string& m) const
  {
    return std::runtime_error("XML parse error at offset " + std::to_string(i_) + ": " + m);
  }
  bool peek(char c) const { return i_ < s_.size() && s_[i_] == c; }
  bool starts(const char* t) const { return s_.compare(i_, std::char_traits<char>::length(t), t) == 0; }
  void ws()
  {
    while (i_ < s_.size() && isspace(static_cast<unsigned char>(s_[i_]))) ++i_;
  }
  void skip_misc()
  {
    for (;;) {
      ws();
      if (starts("<?")) {
        size_t e = s_.find("?>", i_);
        if (e == std::string::npos) throw err("unterminated prolog");
        i_ = e + 2;
      } else if (starts("<!--")) {
        size_t e = s_.find("-->", i_);
        if (e == std::string::npos) throw err("unterminated comment");
        i_ = e + 3;
      } else if (starts("<!DOCTYPE")) {
        size_t e = s_.find('>', i_);
        if (e == std::string::npos) throw err("unterminated doctype");
        i_ = e + 1;
      } else {
        return;
      }
    }
  }
  std::string ident()
  {
    size_t j = i_;
    while (j < s_.size() && (isalnum(static_cast<unsigned char>(s_[j])) || s_[j] == '_' || s_[j] == '-' ||
                              s_[j] == ':' || s_[j] == '.'))
      ++j;
    if (j == i_) throw err("expected a name");
    std::string out = s_.substr(i_, j - i_);
    i_ = j;
    return out;
  }
  static std::string decode(const std::string& t)
  {
    std::string out;
    out.reserve(t.size());
    for (size_t k = 0; k < t.size(); ++k) {
      if (t[k] != '&') {
        out += t[k];
        continue;
      }
      size_t e = t.find(';', k);
      std::string ent = t.substr(k + 1, e - k - 1);
      if (ent == "lt") out += '<';
      else if (ent == "gt") out += '>';
      else if (ent == "amp") out += '&';
      else if (ent == "quot") out += '"';
      else if (ent == "apos") out += '\'';
      else out += "&" + ent + ";";
      k = e;
    }
    return out;
  }
  std::unique_ptr<XmlNode> element()
  {
    auto node = std::make_unique<XmlNode>();
    ++i_;  // '<'
    node->name = ident();
    for (;;) {
      ws();
      if (starts("/>")) {
        i_ += 2;
        return node;
      }
      if (peek('>')) {
        ++i_;
        break;
      }
      std::string k = ident();
      ws();
      if (!peek('=')) throw err("expected '='");
      ++i_;
      ws();
      char q = s_[i_];
      if (q != '"' && q != '\'') throw err("expected quote");
      size_t e = s_.find(q, i_ + 1);
      if (e == std::string::npos) throw err("unterminated attribute");
      node->attrs.emplace_back(k, decode(s_.substr(i_ + 1, e - i_ - 1)));
      i_ = e + 1;
    }
    for (;;) {
      if (i_ >= s_.size()) throw err("unterminated element <" + node->name + ">");
      if (starts("</")) {
        i_ += 2;
        std::string n = ident();
        if (n != node->name) throw err("mismatched </" + n + "> for <" + node->name + ">");
        ws();
        if (!peek('>')) throw err("expected '>'");
        ++i_;
        return node;
      } else if (starts("<!--")) {
        size_t e = s_.find("-->", i_);
        if (e == std::string::npos) throw err("unterminated comment");
        i_ = e + 3;
      } else if (starts("<![CDATA[")) {
        size_t e = s_.find("]]>", i_);
        if (e == std::string::npos) throw err("unterminated CDATA");
        node->text += s_.substr(i_ + 9, e - i_ - 9);
        i_ = e + 3;
      } else if (peek('<')) {
        node->children.push_back(element());
      } else {
        size_t e = s_.find('<', i_);
        if (e == std::string::npos) e = s_.size();
        node->text += decode(s_.substr(i_, e - i_));
        i_ = e;
      }
    }
  }
};

}  // namespace omc
