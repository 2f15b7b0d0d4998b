// INI configuration tree with dune-common ParameterTree semantics.
//
// The reference reads its configuration with Dune::ParameterTreeParser::readINITree plus
// "--key=value" overrides (src/dune_copasi.cc:270-288).  This tree keeps the same reading:
// "[prefix]" headers, "key = value" lines, '#' comments (whole line or rest of a line),
// trimmed keys/values, dotted sub-sections, insertion-ordered sub-keys.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace dcgpu {

class ConfigError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};

class Ini {
 public:
  Ini() = default;
  static Ini parse(const std::string& text);
  // apply "key=value" overrides, one per line
  void apply_overrides(const std::string& lines);

  Ini sub(const std::string& key) const;
  bool has_key(const std::string& key) const;
  bool has_sub(const std::string& key) const;
  std::string get(const std::string& key, const std::string& def) const;
  std::string at(const std::string& key) const;
  double get_double(const std::string& key, double def) const;
  long get_long(const std::string& key, long def) const;
  bool get_bool(const std::string& key, bool def) const;
  std::vector<double> get_doubles(const std::string& key, const std::vector<double>& def) const;
  std::vector<std::string> sub_keys() const;
  void set(const std::string& key, const std::string& value);

 private:
  struct Store {
    std::vector<std::string> order;
    std::map<std::string, std::string> values;
  };
  Ini(std::shared_ptr<Store> s, std::string prefix) : store_(std::move(s)), prefix_(std::move(prefix)) {}
  std::shared_ptr<Store> store_ = std::make_shared<Store>();
  std::string prefix_;
};

std::string trim(const std::string& s);

}  // namespace dcgpu
