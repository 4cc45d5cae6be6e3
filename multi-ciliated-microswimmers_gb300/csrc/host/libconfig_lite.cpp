// Reader/writer for the libconfig text format and the libconfig++ API subset
// declared in libconfig_lite.hpp.  Grammar (libconfig manual, "Configuration
// Files"): settings are `name = value` or `name : value`, terminated by an
// optional `;` or `,`; groups `{...}`, arrays `[...]` (scalars of one type),
// lists `(...)` (any values); integers (decimal or 0x hex, optional L/LL
// suffix), floats, booleans (case-insensitive true/false), double-quoted
// strings with escapes (adjacent literals concatenate); comments `#`, `//`,
// `/* */`; `@include "file"` relative to the including file.
#include "libconfig_lite.hpp"

#include <cctype>
#include <cerrno>
#include <cinttypes>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace libconfig {

// ---------------------------------------------------------------- Setting --

Setting::Setting(Config* cfg, Setting* parent, std::string name, Type type, int line)
    : type_(type), cfg_(cfg), parent_(parent), name_(std::move(name)), line_(line) {}

bool Setting::auto_convert() const { return cfg_ != nullptr && cfg_->auto_convert_; }

void Setting::assert_type(Type want) const {
  if (type_ == want) return;
  bool num_want = want == TypeInt || want == TypeInt64 || want == TypeFloat;
  if (num_want && isNumber() && auto_convert()) return;
  // int <-> int64 always interconvert (libconfig stores large ints as int64)
  if ((want == TypeInt && type_ == TypeInt64) || (want == TypeInt64 && type_ == TypeInt)) return;
  throw SettingTypeException(getPath());
}

std::string Setting::getPath() const {
  if (parent_ == nullptr) return "";
  std::string p = parent_->getPath();
  std::string me;
  if (!name_.empty()) {
    me = name_;
  } else {
    int idx = 0;
    for (size_t i = 0; i < parent_->children_.size(); ++i)
      if (parent_->children_[i].get() == this) idx = (int)i;
    me = "[" + std::to_string(idx) + "]";
  }
  if (p.empty()) return me;
  if (me[0] == '[') return p + me;
  return p + "." + me;
}

Setting& Setting::getParent() const {
  if (parent_ == nullptr) throw SettingNotFoundException("");
  return *parent_;
}

Setting::operator bool() const {
  assert_type(TypeBoolean);
  return bval_;
}

static long long as_int(const Setting& s, double f, long long i, bool is_float) {
  (void)s;
  return is_float ? (long long)f : i;
}

Setting::operator int() const {
  assert_type(TypeInt);
  long long v = as_int(*this, fval_, ival_, type_ == TypeFloat);
  if (v > INT_MAX || v < INT_MIN) throw SettingTypeException(getPath());
  return (int)v;
}
Setting::operator unsigned int() const { return (unsigned int)(int)*this; }
Setting::operator long() const {
  assert_type(TypeInt64);
  return (long)as_int(*this, fval_, ival_, type_ == TypeFloat);
}
Setting::operator unsigned long() const { return (unsigned long)(long)*this; }
Setting::operator long long() const {
  assert_type(TypeInt64);
  return as_int(*this, fval_, ival_, type_ == TypeFloat);
}
Setting::operator unsigned long long() const { return (unsigned long long)(long long)*this; }
Setting::operator double() const {
  assert_type(TypeFloat);
  return type_ == TypeFloat ? fval_ : (double)ival_;
}
Setting::operator float() const { return (float)(double)*this; }
Setting::operator std::string() const {
  assert_type(TypeString);
  return sval_;
}
Setting::operator const char*() const {
  assert_type(TypeString);
  return sval_.c_str();
}

Setting& Setting::operator=(bool v) {
  if (type_ == TypeNone) type_ = TypeBoolean;
  assert_type(TypeBoolean);
  bval_ = v;
  return *this;
}
Setting& Setting::operator=(long long v) {
  if (type_ == TypeNone) type_ = (v > INT_MAX || v < INT_MIN) ? TypeInt64 : TypeInt;
  if (type_ == TypeFloat && auto_convert()) {
    fval_ = (double)v;
    return *this;
  }
  assert_type(TypeInt64);
  if (type_ == TypeInt && (v > INT_MAX || v < INT_MIN)) type_ = TypeInt64;
  ival_ = v;
  return *this;
}
Setting& Setting::operator=(int v) { return *this = (long long)v; }
Setting& Setting::operator=(long v) { return *this = (long long)v; }
Setting& Setting::operator=(double v) {
  if (type_ == TypeNone) type_ = TypeFloat;
  if ((type_ == TypeInt || type_ == TypeInt64) && auto_convert()) {
    ival_ = (long long)v;
    return *this;
  }
  assert_type(TypeFloat);
  fval_ = v;
  return *this;
}
Setting& Setting::operator=(float v) { return *this = (double)v; }
Setting& Setting::operator=(const char* v) {
  if (type_ == TypeNone) type_ = TypeString;
  assert_type(TypeString);
  sval_ = v;
  return *this;
}
Setting& Setting::operator=(const std::string& v) { return *this = v.c_str(); }

Setting* Setting::find_child(const char* name) const {
  if (type_ != TypeGroup) return nullptr;
  for (auto& c : children_)
    if (c->name_ == name) return c.get();
  return nullptr;
}

Setting& Setting::operator[](const char* name) const {
  Setting* c = find_child(name);
  if (c == nullptr) {
    std::string p = getPath();
    throw SettingNotFoundException(p.empty() ? std::string(name) : p + "." + name);
  }
  return *c;
}

Setting& Setting::operator[](int idx) const {
  if (!isAggregate() || idx < 0 || idx >= (int)children_.size())
    throw SettingNotFoundException(getPath() + "[" + std::to_string(idx) + "]");
  return *children_[idx];
}

int Setting::getLength() const { return isAggregate() ? (int)children_.size() : 0; }

bool Setting::exists(const char* name) const { return find_child(name) != nullptr; }

template <typename T>
static bool lookup_into(const Setting& s, const char* name, T& v) {
  if (!s.exists(name)) return false;
  try {
    v = (T)s[name];
    return true;
  } catch (const SettingTypeException&) {
    return false;
  }
}

bool Setting::lookupValue(const char* name, bool& v) const { return lookup_into(*this, name, v); }
bool Setting::lookupValue(const char* name, int& v) const { return lookup_into(*this, name, v); }
bool Setting::lookupValue(const char* name, long long& v) const { return lookup_into(*this, name, v); }
bool Setting::lookupValue(const char* name, double& v) const { return lookup_into(*this, name, v); }
bool Setting::lookupValue(const char* name, float& v) const { return lookup_into(*this, name, v); }
bool Setting::lookupValue(const char* name, std::string& v) const {
  if (!exists(name)) return false;
  const Setting& c = (*this)[name];
  if (c.type_ != TypeString) return false;
  v = c.sval_;
  return true;
}

static bool valid_name(const char* n) {
  if (n == nullptr || !(std::isalpha((unsigned char)n[0]) || n[0] == '*')) return false;
  for (const char* p = n + 1; *p; ++p)
    if (!(std::isalnum((unsigned char)*p) || *p == '_' || *p == '-' || *p == '*')) return false;
  return true;
}

Setting& Setting::add(const char* name, Type type) {
  if (type_ != TypeGroup) throw SettingTypeException(getPath());
  if (!valid_name(name)) throw SettingNameException(getPath() + "." + (name ? name : ""));
  if (find_child(name) != nullptr) throw SettingNameException(getPath() + "." + name);
  children_.emplace_back(new Setting(cfg_, const_cast<Setting*>(this), name, type, 0));
  return *children_.back();
}

Setting& Setting::add(Type type) {
  if (type_ != TypeArray && type_ != TypeList) throw SettingTypeException(getPath());
  if (type_ == TypeArray) {
    if (type >= TypeGroup) throw SettingTypeException(getPath());
    if (!children_.empty() && children_[0]->type_ != type) throw SettingTypeException(getPath());
  }
  children_.emplace_back(new Setting(cfg_, const_cast<Setting*>(this), "", type, 0));
  return *children_.back();
}

void Setting::remove(const char* name) {
  for (size_t i = 0; i < children_.size(); ++i) {
    if (children_[i]->name_ == name) {
      children_.erase(children_.begin() + i);
      return;
    }
  }
  throw SettingNotFoundException(getPath() + "." + name);
}

// ----------------------------------------------------------------- Parser --

namespace {

struct Parser {
  Config* cfg;
  std::string file;
  std::string text;
  size_t pos;
  int line;
  int depth;

  Parser(Config* c, std::string f, std::string t)
      : cfg(c), file(std::move(f)), text(std::move(t)), pos(0), line(1), depth(0) {}

  [[noreturn]] void fail(const std::string& msg) { throw ParseException(file, line, msg); }

  void skip_ws() {
    for (;;) {
      while (pos < text.size() && std::isspace((unsigned char)text[pos])) {
        if (text[pos] == '\n') ++line;
        ++pos;
      }
      if (pos >= text.size()) return;
      if (text[pos] == '#' || (text[pos] == '/' && pos + 1 < text.size() && text[pos + 1] == '/')) {
        while (pos < text.size() && text[pos] != '\n') ++pos;
        continue;
      }
      if (text[pos] == '/' && pos + 1 < text.size() && text[pos + 1] == '*') {
        size_t end = text.find("*/", pos + 2);
        if (end == std::string::npos) fail("unterminated comment");
        for (size_t i = pos; i < end; ++i)
          if (text[i] == '\n') ++line;
        pos = end + 2;
        continue;
      }
      return;
    }
  }

  bool peek(char c) {
    skip_ws();
    return pos < text.size() && text[pos] == c;
  }

  std::string read_name() {
    skip_ws();
    size_t s = pos;
    if (pos < text.size() && (std::isalpha((unsigned char)text[pos]) || text[pos] == '*')) {
      ++pos;
      while (pos < text.size() && (std::isalnum((unsigned char)text[pos]) || text[pos] == '_' ||
                                   text[pos] == '-' || text[pos] == '*'))
        ++pos;
    }
    if (s == pos) fail("syntax error");
    return text.substr(s, pos - s);
  }

  std::string read_string_literal() {
    std::string out;
    for (;;) {
      skip_ws();
      if (pos >= text.size() || text[pos] != '"') break;
      ++pos;
      while (pos < text.size() && text[pos] != '"') {
        char c = text[pos++];
        if (c == '\n') ++line;
        if (c == '\\') {
          if (pos >= text.size()) fail("unterminated string");
          char e = text[pos++];
          switch (e) {
            case 'n': out += '\n'; break;
            case 't': out += '\t'; break;
            case 'r': out += '\r'; break;
            case 'f': out += '\f'; break;
            case '\\': out += '\\'; break;
            case '"': out += '"'; break;
            case 'x': {
              if (pos + 2 > text.size()) fail("bad escape");
              out += (char)std::strtol(text.substr(pos, 2).c_str(), nullptr, 16);
              pos += 2;
              break;
            }
            default: out += e;
          }
        } else {
          out += c;
        }
      }
      if (pos >= text.size()) fail("unterminated string");
      ++pos;  // closing quote; adjacent literals concatenate
    }
    return out;
  }

  // parses a scalar or aggregate value into `s` (whose type is still TypeNone)
  void parse_value(Setting& s) {
    skip_ws();
    if (pos >= text.size()) fail("syntax error");
    char c = text[pos];
    if (c == '{') {
      ++pos;
      s.type_ = Setting::TypeGroup;
      if (++depth > 256) fail("nesting too deep");
      parse_settings(s, '}');
      --depth;
      if (!peek('}')) fail("syntax error");
      ++pos;
      return;
    }
    if (c == '[' || c == '(') {
      char close = c == '[' ? ']' : ')';
      ++pos;
      s.type_ = c == '[' ? Setting::TypeArray : Setting::TypeList;
      if (++depth > 256) fail("nesting too deep");
      bool first = true;
      for (;;) {
        if (peek(close)) {
          ++pos;
          break;
        }
        if (!first) {
          if (!peek(',')) fail("syntax error");
          ++pos;
          if (peek(close)) fail("syntax error");
        }
        first = false;
        std::unique_ptr<Setting> child(new Setting(cfg, &s, "", Setting::TypeNone, line));
        parse_value(*child);
        if (s.type_ == Setting::TypeArray) {
          if (child->isAggregate()) fail("syntax error");
          if (!s.children_.empty()) {
            Setting::Type t0 = s.children_[0]->type_;
            bool ints = (t0 == Setting::TypeInt || t0 == Setting::TypeInt64) &&
                        (child->type_ == Setting::TypeInt || child->type_ == Setting::TypeInt64);
            if (t0 != child->type_ && !ints) fail("mismatched element type in array");
          }
        }
        s.children_.push_back(std::move(child));
      }
      --depth;
      return;
    }
    if (c == '"') {
      s.type_ = Setting::TypeString;
      s.sval_ = read_string_literal();
      return;
    }
    // bool?
    if (std::isalpha((unsigned char)c)) {
      size_t e = pos;
      while (e < text.size() && std::isalpha((unsigned char)text[e])) ++e;
      std::string w = text.substr(pos, e - pos);
      for (auto& ch : w) ch = (char)std::tolower((unsigned char)ch);
      if (w == "true" || w == "false") {
        s.type_ = Setting::TypeBoolean;
        s.bval_ = w == "true";
        pos = e;
        return;
      }
      fail("syntax error");
    }
    // number
    size_t e = pos;
    if (e < text.size() && (text[e] == '+' || text[e] == '-')) ++e;
    if (e + 1 < text.size() && text[e] == '0' && (text[e + 1] == 'x' || text[e + 1] == 'X')) {
      size_t h = e + 2;
      while (h < text.size() && std::isxdigit((unsigned char)text[h])) ++h;
      if (h == e + 2) fail("syntax error");
      std::string num = text.substr(pos, h - pos);
      unsigned long long v = std::strtoull(num.c_str() + (e - pos) + 2, nullptr, 16);
      bool neg = text[pos] == '-';
      long long sv = neg ? -(long long)v : (long long)v;
      pos = h;
      bool l = false;
      while (pos < text.size() && (text[pos] == 'L' || text[pos] == 'l')) {
        ++pos;
        l = true;
      }
      s.type_ = (l || v > 0xffffffffULL) ? Setting::TypeInt64 : Setting::TypeInt;
      if (s.type_ == Setting::TypeInt) sv = (long long)(int)(unsigned int)v;
      s.ival_ = sv;
      return;
    }
    size_t d0 = e;
    while (e < text.size() && std::isdigit((unsigned char)text[e])) ++e;
    bool is_float = false;
    if (e < text.size() && text[e] == '.') {
      is_float = true;
      ++e;
      while (e < text.size() && std::isdigit((unsigned char)text[e])) ++e;
    }
    if (e == d0 || (e == d0 + 1 && is_float)) fail("syntax error");
    if (e < text.size() && (text[e] == 'e' || text[e] == 'E')) {
      size_t x = e + 1;
      if (x < text.size() && (text[x] == '+' || text[x] == '-')) ++x;
      if (x < text.size() && std::isdigit((unsigned char)text[x])) {
        is_float = true;
        e = x;
        while (e < text.size() && std::isdigit((unsigned char)text[e])) ++e;
      }
    }
    std::string num = text.substr(pos, e - pos);
    pos = e;
    if (is_float) {
      s.type_ = Setting::TypeFloat;
      s.fval_ = std::strtod(num.c_str(), nullptr);
      return;
    }
    bool l = false;
    while (pos < text.size() && (text[pos] == 'L' || text[pos] == 'l')) {
      ++pos;
      l = true;
    }
    errno = 0;
    long long v = std::strtoll(num.c_str(), nullptr, 10);
    if (errno == ERANGE) fail("integer value out of range");
    s.type_ = (l || v > INT_MAX || v < INT_MIN) ? Setting::TypeInt64 : Setting::TypeInt;
    s.ival_ = v;
  }

  void parse_settings(Setting& group, char close) {
    for (;;) {
      skip_ws();
      if (pos >= text.size()) {
        if (close == 0) return;
        fail("syntax error");
      }
      if (text[pos] == close) return;
      if (text[pos] == '@') {
        std::string kw = text.substr(pos, 8);
        if (kw != "@include") fail("syntax error");
        pos += 8;
        skip_ws();
        std::string inc = read_string_literal();
        std::string dir;
        size_t slash = file.find_last_of('/');
        if (slash != std::string::npos && !inc.empty() && inc[0] != '/') dir = file.substr(0, slash + 1);
        std::ifstream in(dir + inc);
        if (!in.good()) fail("cannot open include file");
        std::stringstream ss;
        ss << in.rdbuf();
        Parser sub{cfg, dir + inc, ss.str()};
        sub.depth = depth;
        sub.parse_settings(group, 0);
        continue;
      }
      int name_line = line;
      std::string name = read_name();
      skip_ws();
      if (pos >= text.size() || (text[pos] != '=' && text[pos] != ':')) fail("syntax error");
      ++pos;
      for (auto& c : group.children_)
        if (c->getName() != nullptr && name == c->getName()) fail("duplicate setting name");
      std::unique_ptr<Setting> child(new Setting(cfg, &group, name, Setting::TypeNone, name_line));
      parse_value(*child);
      group.children_.push_back(std::move(child));
      skip_ws();
      if (pos < text.size() && (text[pos] == ';' || text[pos] == ',')) ++pos;
    }
  }
};

void write_value(std::ostream& os, const Setting& s, int indent);

void write_indent(std::ostream& os, int indent) {
  for (int i = 0; i < indent; ++i) os << "  ";
}

std::string format_float(double v) {
  char buf[64];
  // shortest representation that reads back to the same double
  for (int prec = 1; prec <= 17; ++prec) {
    std::snprintf(buf, sizeof buf, "%.*g", prec, v);
    if (std::strtod(buf, nullptr) == v) break;
  }
  std::string out(buf);
  if (out.find_first_of(".eEni") == std::string::npos) out += ".0";
  return out;
}

void write_scalar(std::ostream& os, const Setting& s) {
  switch (s.type_) {
    case Setting::TypeInt: os << s.ival_; break;
    case Setting::TypeInt64: os << s.ival_ << "L"; break;
    case Setting::TypeFloat: os << format_float(s.fval_); break;
    case Setting::TypeBoolean: os << (s.bval_ ? "true" : "false"); break;
    case Setting::TypeString: {
      os << '"';
      for (char c : s.sval_) {
        switch (c) {
          case '"': os << "\\\""; break;
          case '\\': os << "\\\\"; break;
          case '\n': os << "\\n"; break;
          case '\t': os << "\\t"; break;
          case '\r': os << "\\r"; break;
          case '\f': os << "\\f"; break;
          default: os << c;
        }
      }
      os << '"';
      break;
    }
    default: break;
  }
}

void write_settings(std::ostream& os, const Setting& g, int indent) {
  for (auto& c : g.children_) {
    write_indent(os, indent);
    os << c->getName() << " = ";
    write_value(os, *c, indent);
    os << ";\n";
  }
}

void write_value(std::ostream& os, const Setting& s, int indent) {
  if (s.type_ == Setting::TypeGroup) {
    os << "{\n";
    write_settings(os, s, indent + 1);
    write_indent(os, indent);
    os << "}";
  } else if (s.type_ == Setting::TypeArray || s.type_ == Setting::TypeList) {
    os << (s.type_ == Setting::TypeArray ? "[ " : "( ");
    for (size_t i = 0; i < s.children_.size(); ++i) {
      if (i) os << ", ";
      write_value(os, *s.children_[i], indent);
    }
    os << (s.type_ == Setting::TypeArray ? " ]" : " )");
  } else {
    write_scalar(os, s);
  }
}

}  // namespace

// ----------------------------------------------------------------- Config --

Config::Config() : root_(new Setting(this, nullptr, "", Setting::TypeGroup, 0)) {}
Config::~Config() = default;

void Config::readFile(const char* filename) {
  std::ifstream in(filename);
  if (!in.good()) throw FileIOException();
  std::stringstream ss;
  ss << in.rdbuf();
  std::unique_ptr<Setting> root(new Setting(this, nullptr, "", Setting::TypeGroup, 0));
  Parser p{this, filename, ss.str()};
  p.parse_settings(*root, 0);
  root_ = std::move(root);
}

void Config::readString(const char* text) {
  std::unique_ptr<Setting> root(new Setting(this, nullptr, "", Setting::TypeGroup, 0));
  Parser p{this, "", text};
  p.parse_settings(*root, 0);
  root_ = std::move(root);
}

std::string Config::writeString() const {
  std::ostringstream os;
  write_settings(os, *root_, 0);
  return os.str();
}

void Config::writeFile(const char* filename) {
  std::ofstream out(filename);
  if (!out.good()) throw FileIOException();
  out << writeString();
  if (!out.good()) throw FileIOException();
}

Setting* Config::find_path(const char* path) const {
  Setting* cur = root_.get();
  std::string p(path);
  size_t i = 0;
  while (i < p.size() && cur != nullptr) {
    if (p[i] == '.' || p[i] == '/' || p[i] == ':') {
      ++i;
      continue;
    }
    if (p[i] == '[') {
      size_t e = p.find(']', i);
      if (e == std::string::npos) return nullptr;
      int idx = std::atoi(p.substr(i + 1, e - i - 1).c_str());
      if (!cur->isAggregate() || idx < 0 || idx >= (int)cur->children_.size()) return nullptr;
      cur = cur->children_[idx].get();
      i = e + 1;
      continue;
    }
    size_t e = p.find_first_of(".[/:", i);
    std::string name = p.substr(i, e == std::string::npos ? std::string::npos : e - i);
    cur = cur->find_child(name.c_str());
    i = e == std::string::npos ? p.size() : e;
  }
  return cur;
}

Setting& Config::lookup(const char* path) const {
  Setting* s = find_path(path);
  if (s == nullptr) throw SettingNotFoundException(path);
  return *s;
}

bool Config::exists(const char* path) const { return find_path(path) != nullptr; }

template <typename T>
static bool cfg_lookup(const Config& c, const char* path, T& v) {
  if (!c.exists(path)) return false;
  try {
    v = (T)c.lookup(path);
    return true;
  } catch (const SettingTypeException&) {
    return false;
  }
}

bool Config::lookupValue(const char* path, double& v) const { return cfg_lookup(*this, path, v); }
bool Config::lookupValue(const char* path, int& v) const { return cfg_lookup(*this, path, v); }
bool Config::lookupValue(const char* path, bool& v) const { return cfg_lookup(*this, path, v); }
bool Config::lookupValue(const char* path, std::string& v) const {
  if (!exists(path)) return false;
  const Setting& s = lookup(path);
  if (s.type_ != Setting::TypeString) return false;
  v = s.sval_;
  return true;
}

}  // namespace libconfig
