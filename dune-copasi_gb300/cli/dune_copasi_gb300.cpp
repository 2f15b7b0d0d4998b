// Thin command-line front end over the C ABI, mirroring the reference CLI
// (src/dune_copasi.cc:139-437): --config=<file> and --key=value options (later ones win),
// --dump-config, --help, --version; then model creation, evolve from time_begin to
// time_end with time_step_initial, VTK output at writer.vtk.path every writer.time_step
// (0: every step, src/dune_copasi.cc:403-418) and the [model.reduce] operators after every
// step (an error flag ends the run with exit code 1, as ReductionError does in the reference).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "dcgpu.h"

namespace {

void help(const char* prog) {
  std::printf(
      "Usage: %s [options]\n"
      "  -h / --help          - Display this help.\n"
      "  --version            - Display the version of this program.\n"
      "  --dump-config        - Print the configuration (file + options) and exit.\n"
      "  --config=<string>    - Configuration file in INI format.\n"
      "  --<key>=<value>      - Set or override a configuration key (e.g. --model.time_step_operator.time_end=1).\n",
      prog);
}

bool get(const dc_model* m, const char* key, std::string* out) {
  char buf[4096];
  if (dc_config_get(m, key, buf, sizeof buf) != DC_OK) return false;
  *out = buf;
  return true;
}

double get_double(const dc_model* m, const char* key, double def) {
  std::string v;
  return get(m, key, &v) ? std::stod(v) : def;
}

struct Writer {
  std::string vtk_path;
  double time_step = 0.0;
  double time_write = 0.0;
  bool first = true;
  bool reduce = false;
  int error = 0;
};

int on_step(const dc_model* m, double t, Writer& w) {
  if (!w.vtk_path.empty() && t >= w.time_write - 1e-9 * w.time_step) {
    if (dc_write_vtk(m, w.vtk_path.c_str(), w.first ? 0 : 1) != DC_OK) {
      std::fprintf(stderr, "VTK output failed: %s\n", dc_last_error());
      return 1;
    }
    w.first = false;
    w.time_write += w.time_step;
  }
  if (w.reduce) {
    size_t n = 0;
    if (dc_reduce(m, nullptr, nullptr, 0, &n) != DC_OK) return 1;
    std::vector<dc_reduce_value> r(n);
    if (dc_reduce(m, nullptr, r.data(), n, &n) != DC_OK) {
      std::fprintf(stderr, "reduce failed: %s\n", dc_last_error());
      return 1;
    }
    for (const auto& v : r) {
      std::printf("  | %s := %.6e |%s\n", v.key, v.value, v.error ? " error" : (v.warn ? " warning" : ""));
      if (v.error) {
        std::fprintf(stderr, "Reduction on the token '%s' raised an error (%s := %.17g)\n", v.key, v.key, v.value);
        return 1;
      }
    }
  }
  return 0;
}

void callback(const dc_model* m, double t, void* user) {
  auto& w = *static_cast<Writer*>(user);
  if (!w.error) w.error = on_step(m, t, w);
}

}  // namespace

int main(int argc, char** argv) {
  std::string cfg_file, overrides;
  bool dump = false;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "-h" || a.rfind("--help", 0) == 0) {
      help(argv[0]);
      return 0;
    }
    if (a == "--version") {
      std::printf("dune-copasi-gb300 (GB300 engine for DuneCopasi models)\n");
      return 0;
    }
    if (a == "--dump-config") {
      dump = true;
    } else if (a.rfind("--config=", 0) == 0) {
      cfg_file = a.substr(9);
    } else if (a.rfind("--", 0) == 0 && a.find('=') != std::string::npos) {
      overrides += a.substr(2) + "\n";
    } else {
      std::fprintf(stderr, "Invalid argument '%s'\n", a.c_str());
      return 1;
    }
  }
  std::string ini;
  if (!cfg_file.empty()) {
    std::ifstream in(cfg_file);
    if (!in) {
      std::fprintf(stderr, "Configuration file '%s' does not exist\n", cfg_file.c_str());
      return 1;
    }
    std::ostringstream ss;
    ss << in.rdbuf();
    ini = ss.str();
  }
  if (dump) {
    std::printf("%s%s", ini.c_str(), overrides.c_str());
    return 0;
  }
  dc_model* m = nullptr;
  if (dc_model_create(ini.c_str(), overrides.empty() ? nullptr : overrides.c_str(), &m) != DC_OK) {
    std::fprintf(stderr, "Invalid configuration: %s\n", dc_last_error());
    return 1;
  }
  Writer w;
  get(m, "model.writer.vtk.path", &w.vtk_path);
  w.time_step = get_double(m, "model.writer.time_step", 0.0);
  size_t nkeys = 0;
  w.reduce = dc_reduce(m, nullptr, nullptr, 0, &nkeys) == DC_OK && nkeys > 0;
  // the initial condition is written and reduced first (src/dune_copasi.cc:428-432)
  double t0 = 0.0;
  dc_state_time(m, &t0);
  w.time_write = t0;
  int rc = on_step(m, t0, w);
  if (rc == 0) {
    const double t_end = get_double(m, "model.time_step_operator.time_end", 1.0);
    double dt_max = get_double(m, "model.time_step_operator.time_step_max", 0.1);
    double dt = get_double(m, "model.time_step_operator.time_step_initial", dt_max);
    const int st = dc_evolve(m, t_end, &dt, callback, &w);
    rc = w.error;
    if (st != DC_OK && rc == 0) {
      std::fprintf(stderr, "Time stepping failed: %s\n", dc_last_error());
      rc = 1;
    }
  }
  dc_model_destroy(m);
  if (rc == 0) std::printf("dune-copasi-gb300 successfully finished :)\n");
  else std::fprintf(stderr, "dune-copasi-gb300 finished with some errors :(\n");
  return rc;
}
