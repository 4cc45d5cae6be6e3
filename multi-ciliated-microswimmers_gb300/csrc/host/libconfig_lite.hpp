// libconfig_lite: a self-contained reader/writer for the libconfig text format
// and the subset of the libconfig++ C++ API that the microswimmer driver uses.
//
// The simulation is configured by `sim.cfg`, a libconfig file
// (src/main.cpp:48-98, src/simulation.cpp:614-673, src/libcilia/global.cpp:21-30,
// src/clami.cpp:32-118, src/cilia.h:11-24, src/sphere.h:14-17).  libconfig++ is
// not available in this toolchain, so this header provides the same class
// names, member functions, conversion operators and exception types:
//
//   Config::readFile / writeFile / getRoot / lookup / exists / lookupValue
//   Setting::operator[](name | index), implicit conversions to
//   int/long long/double/float/bool/std::string, assignment from the same
//   types, getLength, exists, lookupValue, getName, getPath, getType, add.
//
// Type rules follow libconfig: a setting converts only to its own type unless
// auto-conversion is enabled (off by default), int values too large for 32 bits
// are stored as 64-bit, lookupValue never throws (returns false on a missing
// setting or a type mismatch), and operator[] on a missing name or index throws
// SettingNotFoundException.
#pragma once

#include <exception>
#include <memory>
#include <string>
#include <vector>

namespace libconfig {

class Setting;
class Config;

class ConfigException : public std::exception {
 public:
  const char* what() const noexcept override { return "ConfigException"; }
};

class SettingException : public ConfigException {
 public:
  explicit SettingException(std::string path) : path_(std::move(path)) {}
  const char* getPath() const { return path_.c_str(); }
  const char* what() const noexcept override { return "SettingException"; }

 private:
  std::string path_;
};

class SettingTypeException : public SettingException {
 public:
  using SettingException::SettingException;
  const char* what() const noexcept override { return "SettingTypeException"; }
};

class SettingNotFoundException : public SettingException {
 public:
  using SettingException::SettingException;
  const char* what() const noexcept override { return "SettingNotFoundException"; }
};

class SettingNameException : public SettingException {
 public:
  using SettingException::SettingException;
  const char* what() const noexcept override { return "SettingNameException"; }
};

class FileIOException : public ConfigException {
 public:
  const char* what() const noexcept override { return "FileIOException"; }
};

class ParseException : public ConfigException {
 public:
  ParseException(std::string file, int line, std::string error)
      : file_(std::move(file)), line_(line), error_(std::move(error)) {}
  const char* getFile() const { return file_.c_str(); }
  int getLine() const { return line_; }
  const char* getError() const { return error_.c_str(); }
  const char* what() const noexcept override { return "ParseException"; }

 private:
  std::string file_;
  int line_;
  std::string error_;
};

class Setting {
 public:
  enum Type {
    TypeNone = 0,
    TypeInt,
    TypeInt64,
    TypeFloat,
    TypeString,
    TypeBoolean,
    TypeGroup,
    TypeArray,
    TypeList
  };

  Setting(Config* cfg, Setting* parent, std::string name, Type type, int line);
  Setting(const Setting&) = delete;
  Setting& operator=(const Setting&) = delete;

  // value access (libconfig semantics: exact type unless auto-convert is on)
  operator bool() const;
  operator int() const;
  operator unsigned int() const;
  operator long() const;
  operator unsigned long() const;
  operator long long() const;
  operator unsigned long long() const;
  operator double() const;
  operator float() const;
  operator std::string() const;
  operator const char*() const;

  Setting& operator=(bool v);
  Setting& operator=(int v);
  Setting& operator=(long v);
  Setting& operator=(long long v);
  Setting& operator=(double v);
  Setting& operator=(float v);
  Setting& operator=(const char* v);
  Setting& operator=(const std::string& v);

  Setting& operator[](const char* name) const;
  Setting& operator[](const std::string& name) const { return (*this)[name.c_str()]; }
  Setting& operator[](int idx) const;

  bool lookupValue(const char* name, bool& v) const;
  bool lookupValue(const char* name, int& v) const;
  bool lookupValue(const char* name, long long& v) const;
  bool lookupValue(const char* name, double& v) const;
  bool lookupValue(const char* name, float& v) const;
  bool lookupValue(const char* name, std::string& v) const;
  bool lookupValue(const std::string& name, double& v) const { return lookupValue(name.c_str(), v); }
  bool lookupValue(const std::string& name, int& v) const { return lookupValue(name.c_str(), v); }
  bool lookupValue(const std::string& name, std::string& v) const { return lookupValue(name.c_str(), v); }
  bool lookupValue(const std::string& name, bool& v) const { return lookupValue(name.c_str(), v); }

  Setting& add(const char* name, Type type);
  Setting& add(const std::string& name, Type type) { return add(name.c_str(), type); }
  Setting& add(Type type);
  void remove(const char* name);

  bool exists(const char* name) const;
  bool exists(const std::string& name) const { return exists(name.c_str()); }
  int getLength() const;
  Type getType() const { return type_; }
  const char* getName() const { return name_.empty() ? nullptr : name_.c_str(); }
  std::string getPath() const;
  int getSourceLine() const { return line_; }
  bool isGroup() const { return type_ == TypeGroup; }
  bool isArray() const { return type_ == TypeArray; }
  bool isList() const { return type_ == TypeList; }
  bool isAggregate() const { return type_ >= TypeGroup; }
  bool isScalar() const { return type_ > TypeNone && type_ < TypeGroup; }
  bool isNumber() const { return type_ == TypeInt || type_ == TypeInt64 || type_ == TypeFloat; }
  Setting& getParent() const;
  bool isRoot() const { return parent_ == nullptr; }

  // internal access for the reader/writer
  long long ival_ = 0;
  double fval_ = 0.0;
  bool bval_ = false;
  std::string sval_;
  std::vector<std::unique_ptr<Setting>> children_;
  Type type_;

 private:
  friend class Config;
  void assert_type(Type want) const;
  bool auto_convert() const;
  Setting* find_child(const char* name) const;

  Config* cfg_;
  Setting* parent_;
  std::string name_;
  int line_;
};

class Config {
 public:
  Config();
  ~Config();
  Config(const Config&) = delete;
  Config& operator=(const Config&) = delete;

  void readFile(const char* filename);
  void readFile(const std::string& filename) { readFile(filename.c_str()); }
  void readString(const char* text);
  void readString(const std::string& text) { readString(text.c_str()); }
  void writeFile(const char* filename);
  void writeFile(const std::string& filename) { writeFile(filename.c_str()); }
  std::string writeString() const;

  Setting& getRoot() const { return *root_; }
  Setting& lookup(const char* path) const;
  Setting& lookup(const std::string& path) const { return lookup(path.c_str()); }
  bool exists(const char* path) const;
  bool exists(const std::string& path) const { return exists(path.c_str()); }
  bool lookupValue(const char* path, double& v) const;
  bool lookupValue(const char* path, int& v) const;
  bool lookupValue(const char* path, bool& v) const;
  bool lookupValue(const char* path, std::string& v) const;

  void setAutoConvert(bool flag) { auto_convert_ = flag; }
  bool getAutoConvert() const { return auto_convert_; }

 private:
  friend class Setting;
  Setting* find_path(const char* path) const;
  std::unique_ptr<Setting> root_;
  bool auto_convert_ = false;
};

}  // namespace libconfig
