#include "ini.hpp"

#include <algorithm>
#include <cstdlib>
#include <memory>
#include <sstream>

namespace dcgpu {

std::string trim(const std::string& s) {
  size_t b = 0, e = s.size();
  while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
  while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
  return s.substr(b, e - b);
}

Ini Ini::parse(const std::string& text) {
  Ini ini;
  std::istringstream in(text);
  std::string raw, prefix;
  while (std::getline(in, raw)) {
    std::string line = trim(raw);
    if (line.empty() || line[0] == '#') continue;
    if (line[0] == '[') {
      auto end = line.find(']');
      if (end == std::string::npos) throw ConfigError("unterminated section header: " + raw);
      prefix = trim(line.substr(1, end - 1));
      if (!prefix.empty()) prefix += ".";
      continue;
    }
    auto c = line.find('#');
    if (c != std::string::npos) line = line.substr(0, c);
    auto mid = line.find('=');
    if (mid == std::string::npos) continue;
    std::string key = prefix + trim(line.substr(0, mid));
    std::string value = trim(line.substr(mid + 1));
    if (value.size() >= 2 && value.front() == '"' && value.back() == '"')
      value = value.substr(1, value.size() - 2);
    ini.set(key, value);
  }
  return ini;
}

void Ini::apply_overrides(const std::string& lines) {
  std::istringstream in(lines);
  std::string raw;
  while (std::getline(in, raw)) {
    std::string line = trim(raw);
    if (line.rfind("--", 0) == 0) line = line.substr(2);
    if (line.empty()) continue;
    auto mid = line.find('=');
    if (mid == std::string::npos) throw ConfigError("override without '=': " + raw);
    set(trim(line.substr(0, mid)), trim(line.substr(mid + 1)));
  }
}

void Ini::set(const std::string& key, const std::string& value) {
  std::string k = prefix_ + key;
  if (!store_->values.count(k)) store_->order.push_back(k);
  store_->values[k] = value;
}

Ini Ini::sub(const std::string& key) const { return Ini(store_, prefix_ + key + "."); }

bool Ini::has_key(const std::string& key) const { return store_->values.count(prefix_ + key) > 0; }

bool Ini::has_sub(const std::string& key) const {
  std::string p = prefix_ + key + ".";
  for (const auto& k : store_->order)
    if (k.compare(0, p.size(), p) == 0) return true;
  return false;
}

std::string Ini::get(const std::string& key, const std::string& def) const {
  auto it = store_->values.find(prefix_ + key);
  return it == store_->values.end() ? def : it->second;
}

std::string Ini::at(const std::string& key) const {
  auto it = store_->values.find(prefix_ + key);
  if (it == store_->values.end()) throw ConfigError("missing configuration key '" + prefix_ + key + "'");
  return it->second;
}

static double to_double(const std::string& key, const std::string& v) {
  char* end = nullptr;
  std::string t = trim(v);
  double d = std::strtod(t.c_str(), &end);
  if (t.empty() || end == t.c_str() || *end != '\0')
    throw ConfigError("configuration key '" + key + "' is not a number: '" + v + "'");
  return d;
}

double Ini::get_double(const std::string& key, double def) const {
  auto it = store_->values.find(prefix_ + key);
  return it == store_->values.end() ? def : to_double(prefix_ + key, it->second);
}

long Ini::get_long(const std::string& key, long def) const {
  auto it = store_->values.find(prefix_ + key);
  return it == store_->values.end() ? def : static_cast<long>(to_double(prefix_ + key, it->second));
}

bool Ini::get_bool(const std::string& key, bool def) const {
  auto it = store_->values.find(prefix_ + key);
  if (it == store_->values.end()) return def;
  std::string s = trim(it->second);
  std::transform(s.begin(), s.end(), s.begin(), ::tolower);
  if (s == "true" || s == "yes" || s == "on" || s == "1") return true;
  if (s == "false" || s == "no" || s == "off" || s == "0") return false;
  throw ConfigError("configuration key '" + prefix_ + key + "' is not a boolean: '" + it->second + "'");
}

std::vector<double> Ini::get_doubles(const std::string& key, const std::vector<double>& def) const {
  auto it = store_->values.find(prefix_ + key);
  if (it == store_->values.end()) return def;
  std::istringstream in(it->second);
  std::vector<double> out;
  std::string tok;
  while (in >> tok) out.push_back(to_double(prefix_ + key, tok));
  return out;
}

std::vector<std::string> Ini::sub_keys() const {
  std::vector<std::string> out;
  for (const auto& k : store_->order) {
    if (k.compare(0, prefix_.size(), prefix_) != 0) continue;
    std::string rest = k.substr(prefix_.size());
    auto dot = rest.find('.');
    if (dot == std::string::npos) continue;
    std::string head = rest.substr(0, dot);
    if (std::find(out.begin(), out.end(), head) == out.end()) out.push_back(head);
  }
  return out;
}

}  // namespace dcgpu
