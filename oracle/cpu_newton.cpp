// CPU restatement of the reference's implicit step, timed as the CPU baseline (test and
// benchmark infrastructure: never linked into the engine).
//
// What it restates, in C++ with std::thread where the reference runs threads:
//  * structured simplex grid (grid/make_multi_domain_grid.hh:76-91, the Kuhn split of
//    StructuredGridFactory::createSimplexGrid), one compartment covering the domain;
//  * DOF layout: vertex-major, species interleaved
//    (model/diffusion_reaction/model_single_compartment_traits.hh:18-30);
//  * P1 local operator, residual and analytic Jacobian of the mass (storage) and stiffness
//    (reaction, cross diffusion) forms with an order-2 simplex rule
//    (model/diffusion_reaction/local_operator.hh:417-491, 541-707); every functor is one
//    expression evaluated per quadrature point through an interpreted program, as the
//    reference calls its parser per point (model/functor_factory_parser.impl.hh:178-180;
//    constant literals bypass the parser, :125-128);
//  * assembly over colour classes of cells in parallel (the reference's multithreaded
//    PDELab assembler, model/diffusion_reaction/make_step_operator.hh:63-131), into a
//    scalar CSR matrix with the reference's sparsity links (local_operator.hh:276-399);
//  * Newton with the reference's settings (model/make_step_operator.hh:246-288: relative
//    tolerance on the squared l2 norm, iteration range {0, 40}), one-step Runge-Kutta stages
//    in PDELab's parameter form (:408-443);
//  * the linear solve as the reference's iterative default, BiCGSTAB + SSOR (one sweep,
//    relaxation 1; solver/istl/factory/iterative.hh:76-109, preconditioner.hh:226-256),
//    to a relative residual of 1e-10.  SpMV and vector operations use all threads; the SSOR
//    sweeps are sequential, as dune-istl's.  --precond bjacobi replaces SSOR by block Jacobi
//    over the species block of every vertex (the engine's preconditioner; also in the
//    reference's registry), applied with all threads.
//
// Usage:
//   cpu_newton --ini FILE [--state FILE] [--threads T] [--iterations K] [--warmup W]
//              [--steps S] [--out FILE] [--precond ssor|bjacobi] [--time-budget SECONDS]
// With --iterations, the time-stepping sequence runs until W + K Newton iterations are done
// and the last K are timed (with --time-budget, no further timed iteration starts once the
// timed ones have taken that long); with --steps, S whole time steps run and --out receives the
// final state (float64, reference DOF order).  A JSON report goes to stdout.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;
double seconds_since(Clock::time_point t0) {
  return std::chrono::duration<double>(Clock::now() - t0).count();
}

// ------------------------------------------------------------------------ threads
int g_threads = 1;

// f(begin, end, thread) over [0, n) in g_threads contiguous chunks
void parallel_for(int64_t n, const std::function<void(int64_t, int64_t, int)>& f) {
  const int T = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(g_threads, n / 1024 + 1)));
  if (T == 1) {
    f(0, n, 0);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(T);
  for (int t = 0; t < T; ++t) {
    const int64_t b = n * t / T, e = n * (t + 1) / T;
    th.emplace_back([&f, b, e, t] { f(b, e, t); });
  }
  for (auto& x : th) x.join();
}

// ------------------------------------------------------------------------ ini
std::string trim(const std::string& s) {
  size_t b = s.find_first_not_of(" \t\r\n"), e = s.find_last_not_of(" \t\r\n");
  return b == std::string::npos ? "" : s.substr(b, e - b + 1);
}

std::map<std::string, std::string> read_ini(const std::string& text) {
  std::map<std::string, std::string> kv;
  std::istringstream in(text);
  std::string line, section;
  while (std::getline(in, line)) {
    line = trim(line);
    if (line.empty() || line[0] == '#' || line[0] == ';') continue;
    if (line[0] == '[') {
      section = trim(line.substr(1, line.find(']') - 1));
      continue;
    }
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
    if (val.size() >= 2 && (val[0] == '"' || val[0] == '\'') && val.back() == val[0]) val = val.substr(1, val.size() - 2);
    kv[section.empty() ? key : section + "." + key] = val;
  }
  return kv;
}

// ------------------------------------------------------------------------ expressions
// Recursive-descent parser to a stack program (reverse Polish), evaluated per call.
enum Code : uint8_t { C_NUM, C_VAR, C_ADD, C_SUB, C_MUL, C_DIV, C_POW, C_NEG, C_LT, C_LE, C_GT, C_GE, C_EQ, C_NE,
                      C_AND, C_OR, C_SEL, C_FN1, C_FN2, C_POWI };

struct Ins {
  Code code;
  int idx;       // variable slot, or function id
  double value;  // literal
};

class Program {
 public:
  std::vector<Ins> code;
  bool constant = false;
  double cval = 0.0;

  double eval(const double* vars) const {
    if (constant) return cval;
    double st[64];
    int sp = 0;
    for (const Ins& i : code) {
      switch (i.code) {
        case C_NUM: st[sp++] = i.value; break;
        case C_VAR: st[sp++] = vars[i.idx]; break;
        case C_NEG: st[sp - 1] = -st[sp - 1]; break;
        case C_FN1: st[sp - 1] = fn1(i.idx, st[sp - 1]); break;
        case C_POWI: {
          // small integer exponent by multiplication, as the parsers' bytecode optimisers do
          const double a = st[sp - 1];
          double r = 1.0;
          for (int k = 0; k < (i.idx < 0 ? -i.idx : i.idx); ++k) r *= a;
          st[sp - 1] = i.idx < 0 ? 1.0 / r : r;
          break;
        }
        case C_SEL: {
          const double c = st[sp - 3], a = st[sp - 2], b = st[sp - 1];
          sp -= 2;
          st[sp - 1] = c != 0.0 ? a : b;
          break;
        }
        default: {
          const double b = st[--sp], a = st[sp - 1];
          st[sp - 1] = bin(i, a, b);
        }
      }
    }
    return st[0];
  }

 private:
  static double fn1(int f, double a) {
    switch (f) {
      case 0: return std::exp(a);
      case 1: return std::log(a);
      case 2: return std::sqrt(a);
      case 3: return std::fabs(a);
      case 4: return std::sin(a);
      case 5: return std::cos(a);
      case 6: return std::tan(a);
      case 7: return std::tanh(a);
      default: return std::nan("");
    }
  }
  static double bin(const Ins& i, double a, double b) {
    switch (i.code) {
      case C_ADD: return a + b;
      case C_SUB: return a - b;
      case C_MUL: return a * b;
      case C_DIV: return a / b;
      case C_POW: return std::pow(a, b);
      case C_LT: return a < b;
      case C_LE: return a <= b;
      case C_GT: return a > b;
      case C_GE: return a >= b;
      case C_EQ: return a == b;
      case C_NE: return a != b;
      case C_AND: return (a != 0.0 && b != 0.0);
      case C_OR: return (a != 0.0 || b != 0.0);
      case C_FN2:
        return i.idx == 0 ? std::pow(a, b) : i.idx == 1 ? std::min(a, b) : i.idx == 2 ? std::max(a, b)
                                                                                       : std::atan2(a, b);
      default: return std::nan("");
    }
  }
};

class Parser {
 public:
  Parser(const std::string& s, const std::map<std::string, int>& vars, const std::map<std::string, double>& consts)
      : s_(s), vars_(vars), consts_(consts) {}

  Program parse() {
    Program p;
    expr(p.code);
    skip();
    if (pos_ != s_.size()) fail("unexpected '" + s_.substr(pos_) + "'");
    if (p.code.size() == 1 && p.code[0].code == C_NUM) {
      p.constant = true;
      p.cval = p.code[0].value;
    }
    return p;
  }

 private:
  const std::string& s_;
  size_t pos_ = 0;
  const std::map<std::string, int>& vars_;
  const std::map<std::string, double>& consts_;

  [[noreturn]] void fail(const std::string& m) { throw std::runtime_error("expression '" + s_ + "': " + m); }
  void skip() {
    while (pos_ < s_.size() && std::isspace(static_cast<unsigned char>(s_[pos_]))) ++pos_;
  }
  bool eat(const char* t) {
    skip();
    const size_t n = std::strlen(t);
    if (s_.compare(pos_, n, t) == 0) {
      pos_ += n;
      return true;
    }
    return false;
  }
  void expr(std::vector<Ins>& c) {
    orx(c);
    if (eat("?")) {
      expr(c);
      if (!eat(":")) fail("expected ':'");
      expr(c);
      c.push_back({C_SEL, 0, 0.0});
    }
  }
  void orx(std::vector<Ins>& c) {
    andx(c);
    while (eat("||")) {
      andx(c);
      c.push_back({C_OR, 0, 0.0});
    }
  }
  void andx(std::vector<Ins>& c) {
    cmp(c);
    while (eat("&&")) {
      cmp(c);
      c.push_back({C_AND, 0, 0.0});
    }
  }
  void cmp(std::vector<Ins>& c) {
    add(c);
    while (true) {
      Code k;
      if (eat("<=")) k = C_LE;
      else if (eat(">=")) k = C_GE;
      else if (eat("==")) k = C_EQ;
      else if (eat("!=")) k = C_NE;
      else if (eat("<")) k = C_LT;
      else if (eat(">")) k = C_GT;
      else break;
      add(c);
      c.push_back({k, 0, 0.0});
    }
  }
  void add(std::vector<Ins>& c) {
    mul(c);
    while (true) {
      if (eat("+")) {
        mul(c);
        c.push_back({C_ADD, 0, 0.0});
      } else if (eat("-")) {
        mul(c);
        c.push_back({C_SUB, 0, 0.0});
      } else {
        break;
      }
    }
  }
  void mul(std::vector<Ins>& c) {
    unary(c);
    while (true) {
      if (eat("*")) {
        unary(c);
        c.push_back({C_MUL, 0, 0.0});
      } else if (eat("/")) {
        unary(c);
        c.push_back({C_DIV, 0, 0.0});
      } else {
        break;
      }
    }
  }
  void unary(std::vector<Ins>& c) {
    if (eat("-")) {
      unary(c);
      c.push_back({C_NEG, 0, 0.0});
    } else if (eat("+")) {
      unary(c);
    } else {
      power(c);
    }
  }
  void power(std::vector<Ins>& c) {
    primary(c);
    if (eat("^")) {
      std::vector<Ins> e;
      unary(e);
      if (e.size() == 1 && e[0].code == C_NUM && e[0].value == std::floor(e[0].value) && std::fabs(e[0].value) <= 4.0) {
        c.push_back({C_POWI, static_cast<int>(e[0].value), 0.0});
      } else {
        c.insert(c.end(), e.begin(), e.end());
        c.push_back({C_POW, 0, 0.0});
      }
    }
  }
  void primary(std::vector<Ins>& c) {
    skip();
    if (pos_ >= s_.size()) fail("unexpected end");
    const char ch = s_[pos_];
    if (ch == '(') {
      ++pos_;
      expr(c);
      if (!eat(")")) fail("expected ')'");
      return;
    }
    if (std::isdigit(static_cast<unsigned char>(ch)) || ch == '.') {
      char* end = nullptr;
      const double v = std::strtod(s_.c_str() + pos_, &end);
      pos_ = static_cast<size_t>(end - s_.c_str());
      c.push_back({C_NUM, 0, v});
      return;
    }
    if (std::isalpha(static_cast<unsigned char>(ch)) || ch == '_') {
      size_t b = pos_;
      while (pos_ < s_.size() && (std::isalnum(static_cast<unsigned char>(s_[pos_])) || s_[pos_] == '_')) ++pos_;
      const std::string id = s_.substr(b, pos_ - b);
      skip();
      if (pos_ < s_.size() && s_[pos_] == '(') {
        ++pos_;
        static const char* f1[] = {"exp", "log", "sqrt", "abs", "sin", "cos", "tan", "tanh"};
        static const char* f2[] = {"pow", "min", "max", "atan2"};
        for (int k = 0; k < 8; ++k)
          if (id == f1[k]) {
            expr(c);
            if (!eat(")")) fail("expected ')'");
            c.push_back({C_FN1, k, 0.0});
            return;
          }
        for (int k = 0; k < 4; ++k)
          if (id == f2[k]) {
            expr(c);
            if (!eat(",")) fail("expected ','");
            expr(c);
            if (!eat(")")) fail("expected ')'");
            c.push_back({C_FN2, k, 0.0});
            return;
          }
        fail("unknown function " + id);
      }
      auto v = vars_.find(id);
      if (v != vars_.end()) {
        c.push_back({C_VAR, v->second, 0.0});
        return;
      }
      auto k = consts_.find(id);
      if (k != consts_.end()) {
        c.push_back({C_NUM, 0, k->second});
        return;
      }
      fail("unknown symbol " + id);
    }
    fail(std::string("unexpected '") + ch + "'");
  }
};

// an expression is absent when empty or a zero literal (functor_factory_parser.impl.hh:121-124)
bool zero_literal(const std::string& s) {
  const std::string t = trim(s);
  if (t.empty()) return true;
  char* end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  return end && *end == '\0' && v == 0.0;
}

// ------------------------------------------------------------------------ model
struct Pair {
  int w;
  Program f;
};

struct SpeciesEq {
  std::string name;
  bool has_storage = false;
  Program storage;
  std::vector<Pair> storage_jac;
  bool has_reaction = false;
  Program reaction;
  std::vector<Pair> reaction_jac;
  std::vector<Pair> diffusion;  // scalar cross_diffusion.{w}
};

struct Model {
  int dim = 2, ns = 0, nl = 3;
  int64_t nv = 0, ne = 0, ndof = 0;
  std::vector<double> coords;
  std::vector<int64_t> cells;
  std::vector<SpeciesEq> eq;
  std::map<std::string, int> var_slot;  // species values, then time / position
  int slot_time = 0, slot_pos = 0;
  // geometry per cell: |det|, gradients of the basis [nl][dim]
  std::vector<double> adet, grads;
  std::vector<std::vector<int64_t>> colours;
  // CSR
  std::vector<int64_t> rowptr;
  std::vector<int32_t> col;
  // quadrature
  std::vector<double> qp, qw;
  int nq = 0;
};

std::vector<std::string> species_file_order(const std::string& text) {
  std::vector<std::string> out;
  std::istringstream in(text);
  std::string line;
  const std::string pre = "[model.scalar_field.";
  while (std::getline(in, line)) {
    line = trim(line);
    if (line.compare(0, pre.size(), pre) == 0) {
      std::string name = line.substr(pre.size());
      name = name.substr(0, name.find(']'));
      name = name.substr(0, name.find('.'));
      if (std::find(out.begin(), out.end(), name) == out.end()) out.push_back(name);
    }
  }
  return out;
}

void build_mesh(Model& m, const std::map<std::string, std::string>& kv) {
  m.dim = std::stoi(kv.at("grid.dimension"));
  m.nl = m.dim + 1;
  std::vector<int> n(m.dim, 1);
  {
    std::istringstream in(kv.at("grid.cells"));
    for (int d = 0; d < m.dim; ++d) in >> n[d];
  }
  if (kv.count("grid.refinement_level") && std::stoi(kv.at("grid.refinement_level")) != 0)
    throw std::runtime_error("grid.refinement_level is not supported by the CPU restatement");
  if (kv.count("grid.path")) throw std::runtime_error("grid files are not supported by the CPU restatement");
  std::vector<int64_t> npts(m.dim), stride(m.dim);
  m.nv = 1;
  for (int d = 0; d < m.dim; ++d) {
    npts[d] = n[d] + 1;
    stride[d] = m.nv;
    m.nv *= npts[d];
  }
  m.coords.assign(m.nv * m.dim, 0.0);
  for (int64_t v = 0; v < m.nv; ++v) {
    int64_t r = v;
    for (int d = 0; d < m.dim; ++d) {
      const int64_t i = r % npts[d];
      r /= npts[d];
      // numpy.linspace(0, 1, n + 1): i * (1 / n), the last point exactly 1
      m.coords[v * m.dim + d] = (i == n[d]) ? 1.0 : static_cast<double>(i) * (1.0 / n[d]);
    }
  }
  // Kuhn split: per cube (x fastest), one simplex per permutation of the axes in
  // lexicographic order, walking corner 0 -> + e_p0 -> + e_p1 ...
  std::vector<int> perm(m.dim);
  for (int d = 0; d < m.dim; ++d) perm[d] = d;
  std::vector<std::vector<int>> perms;
  do perms.push_back(perm);
  while (std::next_permutation(perm.begin(), perm.end()));
  int64_t ncube = 1;
  for (int d = 0; d < m.dim; ++d) ncube *= n[d];
  m.ne = ncube * static_cast<int64_t>(perms.size());
  m.cells.resize(m.ne * m.nl);
  int64_t e = 0;
  for (int64_t cidx = 0; cidx < ncube; ++cidx) {
    int64_t r = cidx, base = 0;
    for (int d = 0; d < m.dim; ++d) {
      base += (r % n[d]) * stride[d];
      r /= n[d];
    }
    for (const auto& p : perms) {
      int64_t cur = base;
      m.cells[e * m.nl] = cur;
      for (int k = 0; k < m.dim; ++k) {
        cur += stride[p[k]];
        m.cells[e * m.nl + k + 1] = cur;
      }
      ++e;
    }
  }
}

void build_model(Model& m, const std::string& text) {
  const auto kv = read_ini(text);
  build_mesh(m, kv);
  // one compartment covering the domain
  int ncomp = 0;
  for (const auto& [k, v] : kv)
    if (k.compare(0, 13, "compartments.") == 0 && k.size() > 11 &&
        k.compare(k.size() - 11, 11, ".expression") == 0)
      ++ncomp;
  if (ncomp != 1) throw std::runtime_error("the CPU restatement covers one-compartment models only");
  std::map<std::string, double> consts;
  for (const auto& [k, v] : kv) {
    const std::string pre = "parser_context.";
    if (k.compare(0, pre.size(), pre) == 0 && k.size() > 5 && k.compare(k.size() - 5, 5, ".type") == 0) {
      const std::string name = k.substr(pre.size(), k.size() - pre.size() - 5);
      if (v != "constant") throw std::runtime_error("parser_context type " + v + " is not supported");
      consts[name] = std::stod(kv.at(pre + name + ".value"));
    }
  }
  const auto names = species_file_order(text);
  m.ns = static_cast<int>(names.size());
  for (int s = 0; s < m.ns; ++s) m.var_slot[names[s]] = s;
  m.slot_time = m.ns;
  m.slot_pos = m.ns + 1;
  m.var_slot["time"] = m.slot_time;
  const char* ax = "xyz";
  for (int d = 0; d < 3; ++d) m.var_slot[std::string("position_") + ax[d]] = m.slot_pos + d;
  auto get = [&](const std::string& k) -> std::string {
    auto it = kv.find(k);
    return it == kv.end() ? "" : it->second;
  };
  auto compile = [&](const std::string& e) { return Parser(e, m.var_slot, consts).parse(); };
  for (int s = 0; s < m.ns; ++s) {
    SpeciesEq q;
    q.name = names[s];
    const std::string base = "model.scalar_field." + names[s] + ".";
    for (const auto& [k, v] : kv) {
      if (k.compare(0, base.size(), base) != 0) continue;
      const std::string rest = k.substr(base.size());
      if (rest.compare(0, 9, "velocity.") == 0 || rest.compare(0, 8, "outflow.") == 0 ||
          rest.compare(0, 10, "constrain.") == 0)
        if (!zero_literal(v)) throw std::runtime_error("term '" + rest + "' is not supported by the CPU restatement");
    }
    if (!zero_literal(get(base + "storage.expression"))) {
      q.has_storage = true;
      q.storage = compile(get(base + "storage.expression"));
    }
    if (!zero_literal(get(base + "reaction.expression"))) {
      q.has_reaction = true;
      q.reaction = compile(get(base + "reaction.expression"));
    }
    for (int w = 0; w < m.ns; ++w) {
      const std::string sj = get(base + "storage.jacobian." + names[w] + ".expression");
      if (!zero_literal(sj)) q.storage_jac.push_back({w, compile(sj)});
      const std::string rj = get(base + "reaction.jacobian." + names[w] + ".expression");
      if (!zero_literal(rj)) q.reaction_jac.push_back({w, compile(rj)});
      const std::string cd = get(base + "cross_diffusion." + names[w] + ".expression");
      if (!zero_literal(cd)) {
        if (!get(base + "cross_diffusion." + names[w] + ".type").empty() &&
            get(base + "cross_diffusion." + names[w] + ".type") != "scalar")
          throw std::runtime_error("tensor diffusion is not supported by the CPU restatement");
        for (int v = 0; v < m.ns; ++v)
          if (!zero_literal(get(base + "cross_diffusion." + names[w] + ".jacobian." + names[v] + ".expression")))
            throw std::runtime_error("non-linear diffusion is not supported by the CPU restatement");
        q.diffusion.push_back({w, compile(cd)});
      }
    }
    m.eq.push_back(std::move(q));
  }
  m.ndof = m.nv * m.ns;
  // order-2 simplex rules (one point per vertex, symmetric)
  if (m.dim == 2) {
    m.qp = {2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0};
    m.qw = {1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0};
  } else {
    const double a = 0.5854101966249685, b = 0.1381966011250105;
    m.qp = {b, b, b, a, b, b, b, a, b, b, b, a};
    m.qw = {1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0};
  }
  m.nq = static_cast<int>(m.qw.size());
}

void build_geometry(Model& m) {
  const int D = m.dim, L = m.nl;
  m.adet.resize(m.ne);
  m.grads.resize(m.ne * L * D);
  parallel_for(m.ne, [&](int64_t b, int64_t e, int) {
    for (int64_t c = b; c < e; ++c) {
      double B[3][3] = {}, Bi[3][3] = {};
      const int64_t* v = &m.cells[c * L];
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) B[i][j] = m.coords[v[j + 1] * D + i] - m.coords[v[0] * D + i];
      double det;
      if (D == 2) {
        det = B[0][0] * B[1][1] - B[0][1] * B[1][0];
        Bi[0][0] = B[1][1] / det;
        Bi[0][1] = -B[0][1] / det;
        Bi[1][0] = -B[1][0] / det;
        Bi[1][1] = B[0][0] / det;
      } else {
        det = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) - B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
              B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
        Bi[0][0] = (B[1][1] * B[2][2] - B[1][2] * B[2][1]) / det;
        Bi[0][1] = (B[0][2] * B[2][1] - B[0][1] * B[2][2]) / det;
        Bi[0][2] = (B[0][1] * B[1][2] - B[0][2] * B[1][1]) / det;
        Bi[1][0] = (B[1][2] * B[2][0] - B[1][0] * B[2][2]) / det;
        Bi[1][1] = (B[0][0] * B[2][2] - B[0][2] * B[2][0]) / det;
        Bi[1][2] = (B[0][2] * B[1][0] - B[0][0] * B[1][2]) / det;
        Bi[2][0] = (B[1][0] * B[2][1] - B[1][1] * B[2][0]) / det;
        Bi[2][1] = (B[0][1] * B[2][0] - B[0][0] * B[2][1]) / det;
        Bi[2][2] = (B[0][0] * B[1][1] - B[0][1] * B[1][0]) / det;
      }
      m.adet[c] = std::fabs(det);
      // physical gradients: reference gradient of vertex a times B^{-1}
      double* G = &m.grads[c * L * D];
      for (int j = 0; j < D; ++j) {
        double s = 0.0;
        for (int k = 0; k < D; ++k) {
          G[(k + 1) * D + j] = Bi[k][j];
          s += Bi[k][j];
        }
        G[j] = -s;
      }
    }
  });
}

// greedy colouring of the cells (cells of one colour share no vertex), cells of a colour
// in ascending order
void build_colours(Model& m) {
  const int L = m.nl;
  std::vector<int> colour(m.ne, -1);
  std::vector<uint64_t> used(m.nv, 0);  // bit c: a cell of colour c touches the vertex
  int ncol = 0;
  for (int64_t c = 0; c < m.ne; ++c) {
    uint64_t u = 0;
    for (int a = 0; a < L; ++a) u |= used[m.cells[c * L + a]];
    int k = 0;
    while (k < 64 && ((u >> k) & 1)) ++k;
    if (k == 64) throw std::runtime_error("colouring needs more than 64 colours");
    colour[c] = k;
    ncol = std::max(ncol, k + 1);
    for (int a = 0; a < L; ++a) used[m.cells[c * L + a]] |= uint64_t{1} << k;
  }
  m.colours.assign(ncol, {});
  for (int64_t c = 0; c < m.ne; ++c) m.colours[colour[c]].push_back(c);
}

// scalar CSR pattern: row (vertex a, species s) links (vertex b, species w) when s's
// storage, storage Jacobian, reaction Jacobian or cross diffusion names w
// (local_operator.hh:276-399); rows sorted by column
void build_pattern(Model& m) {
  const int L = m.nl, S = m.ns;
  std::vector<std::vector<char>> link(S, std::vector<char>(S, 0));
  for (int s = 0; s < S; ++s) {
    const auto& q = m.eq[s];
    if (q.has_storage) link[s][s] = 1;
    for (const auto& p : q.storage_jac) link[s][p.w] = 1;
    for (const auto& p : q.reaction_jac) link[s][p.w] = 1;
    for (const auto& p : q.diffusion) link[s][p.w] = 1;
  }
  // vertex adjacency (including self)
  std::vector<std::vector<int64_t>> adj(m.nv);
  for (int64_t c = 0; c < m.ne; ++c)
    for (int a = 0; a < L; ++a)
      for (int b = 0; b < L; ++b) adj[m.cells[c * L + a]].push_back(m.cells[c * L + b]);
  m.rowptr.assign(m.ndof + 1, 0);
  std::vector<std::vector<int64_t>> vcols(m.nv);
  for (int64_t v = 0; v < m.nv; ++v) {
    auto& a = adj[v];
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  for (int64_t v = 0; v < m.nv; ++v)
    for (int s = 0; s < S; ++s) {
      int64_t cnt = 0;
      for (int w = 0; w < S; ++w) cnt += link[s][w];
      m.rowptr[v * S + s + 1] = cnt * static_cast<int64_t>(adj[v].size());
    }
  for (int64_t i = 0; i < m.ndof; ++i) m.rowptr[i + 1] += m.rowptr[i];
  m.col.resize(m.rowptr[m.ndof]);
  for (int64_t v = 0; v < m.nv; ++v)
    for (int s = 0; s < S; ++s) {
      int64_t p = m.rowptr[v * S + s];
      for (int64_t b : adj[v])
        for (int w = 0; w < S; ++w)
          if (link[s][w]) m.col[p++] = static_cast<int32_t>(b * S + w);
    }
}

int64_t find_col(const Model& m, int64_t row, int64_t c) {
  const int32_t* b = m.col.data() + m.rowptr[row];
  const int32_t* e = m.col.data() + m.rowptr[row + 1];
  const int32_t* p = std::lower_bound(b, e, static_cast<int32_t>(c));
  if (p == e || *p != c) throw std::runtime_error("pattern lacks an entry");
  return p - m.col.data();
}

// r += cm M(x) + ca A(x) and (J non-null) J += cm dM/dx + ca dA/dx over all cells, the
// cells of each colour in parallel.  Every functor is evaluated at every quadrature point;
// the point contributions to the element matrix are summed per species pair first (mass
// type: one weight per point, diffusion: one coefficient, the basis products being
// constant tables / constant on a P1 cell) and the element matrix formed once per cell.
constexpr int kMaxS = 16, kMaxL = 4, kMaxQ = 4;

void assemble(const Model& m, const std::vector<double>& x, double t, double cm, double ca, double* r, double* J) {
  const int D = m.dim, L = m.nl, S = m.ns, NQ = m.nq;
  if (S > kMaxS) throw std::runtime_error("more species than the CPU restatement supports");
  // basis values and their products at the points
  double phi[kMaxQ][kMaxL], pp[kMaxQ][kMaxL][kMaxL];
  for (int q = 0; q < NQ; ++q) {
    double sum = 0.0;
    for (int k = 0; k < D; ++k) {
      phi[q][k + 1] = m.qp[q * D + k];
      sum += m.qp[q * D + k];
    }
    phi[q][0] = 1.0 - sum;
    for (int a = 0; a < L; ++a)
      for (int b = 0; b < L; ++b) pp[q][a][b] = phi[q][a] * phi[q][b];
  }
  for (const auto& cells : m.colours) {
    parallel_for(static_cast<int64_t>(cells.size()), [&](int64_t b0, int64_t e0, int) {
      std::vector<double> vars(m.ns + 4, 0.0);
      double c[kMaxL][kMaxS], rl[kMaxL][kMaxS], u[kMaxS], g[kMaxS][3];
      std::vector<double> mw(S * S * NQ), dc(S * S);
      std::vector<char> mused(S * S), dused(S * S);
      for (int64_t ci = b0; ci < e0; ++ci) {
        const int64_t cell = cells[ci];
        const int64_t* v = &m.cells[cell * L];
        const double* G = &m.grads[cell * L * D];
        const double adet = m.adet[cell];
        for (int a = 0; a < L; ++a)
          for (int s = 0; s < S; ++s) {
            c[a][s] = x[v[a] * S + s];
            rl[a][s] = 0.0;
          }
        if (J) {
          std::fill(mw.begin(), mw.end(), 0.0);
          std::fill(dc.begin(), dc.end(), 0.0);
          std::fill(mused.begin(), mused.end(), 0);
          std::fill(dused.begin(), dused.end(), 0);
        }
        // species gradients and gradient products of the basis (constant on a P1 cell)
        double GG[kMaxL][kMaxL];
        for (int a = 0; a < L; ++a)
          for (int bb = 0; bb < L; ++bb) {
            double gg = 0.0;
            for (int j = 0; j < D; ++j) gg += G[bb * D + j] * G[a * D + j];
            GG[a][bb] = gg;
          }
        for (int s = 0; s < S; ++s)
          for (int j = 0; j < D; ++j) {
            double acc = 0.0;
            for (int a = 0; a < L; ++a) acc += c[a][s] * G[a * D + j];
            g[s][j] = acc;
          }
        // grad u_w . grad phi_a, also constant on the cell
        double gG[kMaxS][kMaxL];
        if (r)
          for (int w = 0; w < S; ++w)
            for (int a = 0; a < L; ++a) {
              double gg = 0.0;
              for (int j = 0; j < D; ++j) gg += g[w][j] * G[a * D + j];
              gG[w][a] = gg;
            }
        for (int q = 0; q < NQ; ++q) {
          const double fq = m.qw[q] * adet;
          for (int s = 0; s < S; ++s) {
            double acc = 0.0;
            for (int a = 0; a < L; ++a) acc += c[a][s] * phi[q][a];
            u[s] = acc;
            vars[s] = acc;
          }
          vars[m.slot_time] = t;
          for (int d = 0; d < 3; ++d) {
            double acc = 0.0;
            if (d < D)
              for (int a = 0; a < L; ++a) acc += m.coords[v[a] * D + d] * phi[q][a];
            vars[m.slot_pos + d] = acc;
          }
          for (int s = 0; s < S; ++s) {
            const SpeciesEq& eq = m.eq[s];
            double scal = 0.0;  // residual: scalar part at the point (times phi_a)
            // mass form: storage(u) u_s phi_a
            if (cm != 0.0 && eq.has_storage) {
              const double st = eq.storage.eval(vars.data());
              scal += cm * u[s] * st;
              if (J) {
                mw[(s * S + s) * NQ + q] += cm * st * fq;
                mused[s * S + s] = 1;
                for (const auto& p : eq.storage_jac) {
                  mw[(s * S + p.w) * NQ + q] += cm * p.f.eval(vars.data()) * u[s] * fq;
                  mused[s * S + p.w] = 1;
                }
              }
            }
            if (ca != 0.0) {
              // stiffness form: - reaction phi_a + (D_w grad u_w) . grad phi_a
              if (eq.has_reaction) {
                if (r) scal -= ca * eq.reaction.eval(vars.data());
                if (J)
                  for (const auto& p : eq.reaction_jac) {
                    mw[(s * S + p.w) * NQ + q] -= ca * p.f.eval(vars.data()) * fq;
                    mused[s * S + p.w] = 1;
                  }
              }
              for (const auto& p : eq.diffusion) {
                const double dv = p.f.eval(vars.data());
                if (r) {
                  const double k = ca * dv * fq;
                  for (int a = 0; a < L; ++a) rl[a][s] += k * gG[p.w][a];
                }
                if (J) {
                  dc[s * S + p.w] += ca * dv * fq;
                  dused[s * S + p.w] = 1;
                }
              }
            }
            if (r && scal != 0.0)
              for (int a = 0; a < L; ++a) rl[a][s] += scal * phi[q][a] * fq;
          }
        }
        // scatter (cells of one colour share no vertex: no two threads touch a row)
        for (int a = 0; a < L; ++a)
          for (int s = 0; s < S; ++s) {
            const int64_t row = v[a] * S + s;
            if (r) r[row] += rl[a][s];
            if (!J) continue;
            for (int bb = 0; bb < L; ++bb) {
              int64_t p = find_col(m, row, v[bb] * S);
              const int64_t pend = m.rowptr[row + 1];
              for (int w = 0; w < S; ++w) {
                const int k = s * S + w;
                if (!mused[k] && !dused[k]) continue;
                double val = 0.0;
                if (mused[k])
                  for (int q = 0; q < NQ; ++q) val += mw[k * NQ + q] * pp[q][a][bb];
                if (dused[k]) val += dc[k] * GG[a][bb];
                // the row holds (vertex b, w) for every linked w, ascending
                while (p < pend && m.col[p] < v[bb] * S + w) ++p;
                if (p < pend && m.col[p] == v[bb] * S + w) J[p] += val;
                else if (val != 0.0) throw std::runtime_error("pattern lacks an entry");
              }
            }
          }
      }
    });
  }
}

// ------------------------------------------------------------------------ linear algebra
double dot(const std::vector<double>& a, const std::vector<double>& b) {
  std::vector<double> part(g_threads, 0.0);
  parallel_for(static_cast<int64_t>(a.size()), [&](int64_t s, int64_t e, int t) {
    double acc = 0.0;
    for (int64_t i = s; i < e; ++i) acc += a[i] * b[i];
    part[t] = acc;
  });
  double acc = 0.0;
  for (double p : part) acc += p;
  return acc;
}

void spmv(const Model& m, const std::vector<double>& A, const std::vector<double>& x, std::vector<double>& y) {
  parallel_for(m.ndof, [&](int64_t s, int64_t e, int) {
    for (int64_t i = s; i < e; ++i) {
      double acc = 0.0;
      for (int64_t p = m.rowptr[i]; p < m.rowptr[i + 1]; ++p) acc += A[p] * x[m.col[p]];
      y[i] = acc;
    }
  });
}

enum class Precond { SSOR, BlockJacobi };
Precond g_precond = Precond::SSOR;

// inverse of the species block of every vertex (block Jacobi, the preconditioner of the
// engine's solve), one block per vertex, all threads
void block_inverses(const Model& m, const std::vector<double>& A, std::vector<double>& inv) {
  const int S = m.ns;
  inv.resize(m.nv * S * S);
  parallel_for(m.nv, [&](int64_t b, int64_t e, int) {
    std::vector<double> blk(S * 2 * S);
    for (int64_t v = b; v < e; ++v) {
      // [block | I] -> [I | block^-1] by Gauss-Jordan with partial pivoting
      for (int i = 0; i < S; ++i) {
        const int64_t row = v * S + i;
        for (int j = 0; j < 2 * S; ++j) blk[i * 2 * S + j] = (j - S == i) ? 1.0 : 0.0;
        for (int64_t p = m.rowptr[row]; p < m.rowptr[row + 1]; ++p) {
          const int64_t cc = m.col[p];
          if (cc >= v * S && cc < (v + 1) * S) blk[i * 2 * S + (cc - v * S)] = A[p];
        }
      }
      for (int k = 0; k < S; ++k) {
        int piv = k;
        for (int i = k + 1; i < S; ++i)
          if (std::fabs(blk[i * 2 * S + k]) > std::fabs(blk[piv * 2 * S + k])) piv = i;
        if (piv != k)
          for (int j = 0; j < 2 * S; ++j) std::swap(blk[k * 2 * S + j], blk[piv * 2 * S + j]);
        const double d = blk[k * 2 * S + k];
        for (int j = 0; j < 2 * S; ++j) blk[k * 2 * S + j] /= d;
        for (int i = 0; i < S; ++i) {
          if (i == k) continue;
          const double f = blk[i * 2 * S + k];
          if (f != 0.0)
            for (int j = 0; j < 2 * S; ++j) blk[i * 2 * S + j] -= f * blk[k * 2 * S + j];
        }
      }
      for (int i = 0; i < S; ++i)
        for (int j = 0; j < S; ++j) inv[(v * S + i) * S + j] = blk[i * 2 * S + S + j];
    }
  });
}

void block_jacobi(const Model& m, const std::vector<double>& inv, const std::vector<double>& r, std::vector<double>& z) {
  const int S = m.ns;
  parallel_for(m.nv, [&](int64_t b, int64_t e, int) {
    for (int64_t v = b; v < e; ++v)
      for (int i = 0; i < S; ++i) {
        double acc = 0.0;
        for (int j = 0; j < S; ++j) acc += inv[(v * S + i) * S + j] * r[v * S + j];
        z[v * S + i] = acc;
      }
  });
}

// SSOR preconditioner, one symmetric sweep with relaxation 1 from z = 0 (sequential)
void ssor(const Model& m, const std::vector<double>& A, const std::vector<int64_t>& diag, const std::vector<double>& r,
          std::vector<double>& z) {
  const int64_t n = m.ndof;
  for (int64_t i = 0; i < n; ++i) {
    double acc = r[i];
    for (int64_t p = m.rowptr[i]; p < diag[i]; ++p) acc -= A[p] * z[m.col[p]];
    z[i] = acc / A[diag[i]];
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double acc = 0.0;
    for (int64_t p = diag[i] + 1; p < m.rowptr[i + 1]; ++p) acc += A[p] * z[m.col[p]];
    z[i] -= acc / A[diag[i]];
  }
}

// BiCGSTAB + SSOR (or block Jacobi): solves A z = b to |b - A z| <= rel |b|; returns the
// iterations
int bicgstab(const Model& m, const std::vector<double>& A, const std::vector<int64_t>& diag,
             const std::vector<double>& b, std::vector<double>& z, double rel, int max_it) {
  const int64_t n = m.ndof;
  std::vector<double> inv;
  if (g_precond == Precond::BlockJacobi) block_inverses(m, A, inv);
  auto precond = [&](const std::vector<double>& in, std::vector<double>& out) {
    if (g_precond == Precond::BlockJacobi) block_jacobi(m, inv, in, out);
    else ssor(m, A, diag, in, out);
  };
  std::vector<double> r(b), rh(b), p(n, 0.0), v(n, 0.0), s(n), t(n), ph(n), sh(n);
  std::fill(z.begin(), z.end(), 0.0);
  const double bn = std::sqrt(dot(b, b));
  if (bn == 0.0) return 0;
  double rho = 1.0, alpha = 1.0, omega = 1.0;
  for (int it = 1; it <= max_it; ++it) {
    const double rho1 = dot(rh, r);
    const double beta = (rho1 / rho) * (alpha / omega);
    rho = rho1;
    parallel_for(n, [&](int64_t a, int64_t e, int) {
      for (int64_t i = a; i < e; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
    });
    precond(p, ph);
    spmv(m, A, ph, v);
    alpha = rho / dot(rh, v);
    parallel_for(n, [&](int64_t a, int64_t e, int) {
      for (int64_t i = a; i < e; ++i) s[i] = r[i] - alpha * v[i];
    });
    precond(s, sh);
    spmv(m, A, sh, t);
    omega = dot(t, s) / dot(t, t);
    parallel_for(n, [&](int64_t a, int64_t e, int) {
      for (int64_t i = a; i < e; ++i) {
        z[i] += alpha * ph[i] + omega * sh[i];
        r[i] = s[i] - omega * t[i];
      }
    });
    if (std::sqrt(dot(r, r)) <= rel * bn) return it;
    if (!std::isfinite(omega) || omega == 0.0) throw std::runtime_error("BiCGSTAB breakdown");
  }
  throw std::runtime_error("BiCGSTAB did not converge");
}

// ------------------------------------------------------------------------ time stepping
struct Scheme {
  std::vector<std::vector<double>> A, B;
  std::vector<double> D;
};

Scheme scheme(const std::string& name) {
  Scheme s;
  if (name == "ImplicitEuler") {
    s.A = {{-1.0, 1.0}};
    s.B = {{0.0, 1.0}};
    s.D = {0.0, 1.0};
  } else if (name == "Alexander2") {
    const double a = 1.0 - 0.5 * std::sqrt(2.0);
    s.A = {{-1.0, 1.0, 0.0}, {-1.0, 0.0, 1.0}};
    s.B = {{0.0, a, 0.0}, {0.0, 1.0 - a, a}};
    s.D = {0.0, a, 1.0};
  } else {
    throw std::runtime_error("time stepping type " + name + " is not supported by the CPU restatement");
  }
  return s;
}

struct Report {
  int64_t newton = 0, timed_newton = 0, krylov = 0;
  double seconds = 0.0, asm_seconds = 0.0, solve_seconds = 0.0;
  std::vector<int> newton_per_stage;
};

struct Stepper {
  const Model& m;
  double rel = 1e-4;
  int it_max = 40;
  int64_t budget = -1;  // stop after this many Newton iterations (-1: no limit)
  int64_t warmup = 0;
  Report rep;
  std::vector<double> J;
  std::vector<int64_t> diag;
  Clock::time_point mark, last;
  bool timing = false;

  explicit Stepper(const Model& mm) : m(mm) {
    J.resize(m.col.size());
    diag.resize(m.ndof);
    for (int64_t i = 0; i < m.ndof; ++i) diag[i] = find_col(m, i, i);
  }

  double time_budget = -1.0;  // seconds of timed iterations after which no new one starts (-1: none)

  bool done() const {
    if (budget >= 0 && rep.newton >= warmup + budget) return true;
    // a time budget ends the timed region after at least one timed iteration
    return time_budget > 0.0 && rep.timed_newton > 0 &&
           std::chrono::duration<double>(last - mark).count() >= time_budget;
  }

  // iteration boundary: the Newton iteration just finished counts as timed once the
  // warm-up iterations are done
  void tick(double asm_s, double solve_s) {
    ++rep.newton;
    if (rep.newton == warmup) {
      mark = Clock::now();
      timing = true;
      return;
    }
    if (timing) {
      ++rep.timed_newton;
      rep.asm_seconds += asm_s;
      rep.solve_seconds += solve_s;
      last = Clock::now();
    }
  }

  // one time step; false when the iteration budget ran out inside it
  bool step(std::vector<double>& x, double t, double dt, const Scheme& sc) {
    const int ns = static_cast<int>(sc.A.size());
    std::vector<std::vector<double>> us{x};
    std::vector<double> y = x, r(m.ndof), z(m.ndof), cst(m.ndof);
    if (warmup == 0 && !timing) {
      mark = Clock::now();
      timing = true;
    }
    for (int i = 1; i <= ns; ++i) {
      const auto& a = sc.A[i - 1];
      const auto& b = sc.B[i - 1];
      std::fill(cst.begin(), cst.end(), 0.0);
      auto t0 = Clock::now();
      for (int j = 0; j < i; ++j)
        if (a[j] != 0.0 || b[j] != 0.0) assemble(m, us[j], t + sc.D[j] * dt, a[j], b[j] * dt, cst.data(), nullptr);
      const double ai = a[i], bi = b[i] * dt, ti = t + sc.D[i] * dt;
      auto residual = [&](const std::vector<double>& v) {
        r = cst;
        assemble(m, v, ti, ai, bi, r.data(), nullptr);
      };
      residual(y);
      double pending_asm = seconds_since(t0);
      double defect = dot(r, r);  // squared l2 norm (make_step_operator.hh:274-276)
      const double first = defect;
      int it = 0;
      while (true) {
        if (!std::isfinite(defect)) throw std::runtime_error("Newton defect is not finite");
        if (defect < first * rel || defect == 0.0) break;
        if (it >= it_max) throw std::runtime_error("Newton did not converge");
        if (done()) return false;
        auto ta = Clock::now();
        std::fill(J.begin(), J.end(), 0.0);
        assemble(m, y, ti, ai, bi, nullptr, J.data());
        double asm_s = pending_asm + seconds_since(ta);
        auto ts = Clock::now();
        const int k = bicgstab(m, J, diag, r, z, 1e-10, 5000);
        const double solve_s = seconds_since(ts);
        if (timing) rep.krylov += k;
        for (int64_t q = 0; q < m.ndof; ++q) y[q] -= z[q];
        auto tr = Clock::now();
        residual(y);
        asm_s += seconds_since(tr);
        pending_asm = 0.0;
        defect = dot(r, r);
        ++it;
        tick(asm_s, solve_s);
      }
      rep.newton_per_stage.push_back(it);
      us.push_back(y);
    }
    x = y;
    return true;
  }
};

// the host CPU: x86 "model name", or on Arm the implementer and part numbers (Neoverse V2,
// the Grace core, is implementer 0x41 part 0xd4f)
std::string cpu_name() {
  std::ifstream in("/proc/cpuinfo");
  std::string line, implementer, part;
  auto value = [&]() { return trim(line.substr(line.find(':') + 1)); };
  while (std::getline(in, line)) {
    if (line.compare(0, 10, "model name") == 0) return value();
    if (implementer.empty() && line.compare(0, 15, "CPU implementer") == 0) implementer = value();
    if (part.empty() && line.compare(0, 8, "CPU part") == 0) part = value();
  }
  if (part.empty()) return "";
  std::string name = "CPU implementer " + implementer + " part " + part;
  if (implementer == "0x41" && part == "0xd4f") name += " (Arm Neoverse V2)";
  return name;
}

}  // namespace

int main(int argc, char** argv) {
  std::string ini_path, state_path, out_path;
  int64_t iterations = -1, warmup = 0, steps = -1;
  double time_budget = -1.0;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) throw std::runtime_error("missing value for " + a);
      return argv[++i];
    };
    if (a == "--ini") ini_path = next();
    else if (a == "--state") state_path = next();
    else if (a == "--out") out_path = next();
    else if (a == "--threads") g_threads = std::max(1, std::stoi(next()));
    else if (a == "--iterations") iterations = std::stoll(next());
    else if (a == "--warmup") warmup = std::stoll(next());
    else if (a == "--steps") steps = std::stoll(next());
    else if (a == "--time-budget") time_budget = std::stod(next());
    else if (a == "--precond") {
      const std::string v = next();
      if (v == "ssor") g_precond = Precond::SSOR;
      else if (v == "bjacobi") g_precond = Precond::BlockJacobi;
      else throw std::runtime_error("--precond must be ssor or bjacobi");
    }
    else {
      std::fprintf(stderr, "unknown option %s\n", a.c_str());
      return 2;
    }
  }
  try {
    std::ifstream f(ini_path);
    if (!f) throw std::runtime_error("cannot read " + ini_path);
    std::stringstream buf;
    buf << f.rdbuf();
    const std::string text = buf.str();
    const auto kv = read_ini(text);
    Model m;
    auto t_setup = Clock::now();
    build_model(m, text);
    build_geometry(m);
    build_colours(m);
    build_pattern(m);
    const double setup_s = seconds_since(t_setup);
    std::vector<double> x(m.ndof, 0.0);
    if (!state_path.empty()) {
      std::ifstream sf(state_path, std::ios::binary);
      sf.read(reinterpret_cast<char*>(x.data()), m.ndof * sizeof(double));
      if (sf.gcount() != static_cast<std::streamsize>(m.ndof * sizeof(double)))
        throw std::runtime_error("state file holds fewer than n_dof values");
    } else {
      // nodal interpolation of initial.expression at time_begin (model/make_initial.hh:24-90)
      std::map<std::string, double> consts;
      for (const auto& [k, v] : kv) {
        const std::string pre = "parser_context.";
        if (k.compare(0, pre.size(), pre) == 0 && k.size() > 5 && k.compare(k.size() - 5, 5, ".type") == 0) {
          const std::string name = k.substr(pre.size(), k.size() - pre.size() - 5);
          consts[name] = std::stod(kv.at(pre + name + ".value"));
        }
      }
      const double t0 = kv.count("model.time_step_operator.time_begin")
                            ? std::stod(kv.at("model.time_step_operator.time_begin")) : 0.0;
      std::vector<double> vars(m.ns + 4, 0.0);
      for (int s = 0; s < m.ns; ++s) {
        auto it = kv.find("model.scalar_field." + m.eq[s].name + ".initial.expression");
        if (it == kv.end() || zero_literal(it->second)) continue;
        const Program p = Parser(it->second, m.var_slot, consts).parse();
        for (int64_t v = 0; v < m.nv; ++v) {
          vars[m.slot_time] = t0;
          for (int d = 0; d < 3; ++d) vars[m.slot_pos + d] = d < m.dim ? m.coords[v * m.dim + d] : 0.0;
          x[v * m.ns + s] = p.eval(vars.data());
        }
      }
    }
    auto get = [&](const std::string& k, const std::string& d) {
      auto it = kv.find(k);
      return it == kv.end() ? d : it->second;
    };
    const std::string tso = "model.time_step_operator.";
    const Scheme sc = scheme(get(tso + "type", "Alexander2"));
    const double dt = std::stod(get(tso + "time_step_initial", "0.1"));
    double t = std::stod(get(tso + "time_begin", "0"));
    Stepper st(m);
    st.rel = std::stod(get(tso + "nonlinear_solver.convergence_condition.relative_tolerance", "1e-4"));
    st.budget = iterations;
    st.time_budget = time_budget;
    st.warmup = warmup;
    int64_t nsteps = 0;
    while (true) {
      if (steps >= 0 && nsteps >= steps) break;
      if (!st.step(x, t, dt, sc)) break;
      t += dt;
      ++nsteps;
      if (iterations >= 0 && st.done()) break;
    }
    st.rep.seconds = st.rep.timed_newton > 0 ? std::chrono::duration<double>(st.last - st.mark).count() : 0.0;
    if (!out_path.empty()) {
      std::ofstream of(out_path, std::ios::binary);
      of.write(reinterpret_cast<const char*>(x.data()), m.ndof * sizeof(double));
    }
    const Report& r = st.rep;
    const double value = r.seconds > 0 ? static_cast<double>(m.ndof) * r.timed_newton / r.seconds : 0.0;
    std::printf("{\"ndof\": %lld, \"cells\": %lld, \"colours\": %zu, \"nnz\": %zu, \"threads\": %d, "
                "\"setup_seconds\": %.6f, \"steps\": %lld, \"newton_iterations\": %lld, "
                "\"timed_newton_iterations\": %lld, \"seconds\": %.6f, \"assembly_seconds\": %.6f, "
                "\"solve_seconds\": %.6f, \"krylov_iterations\": %lld, \"value\": %.6f, \"cpu\": \"%s\", \"precond\": \"%s\", "
                "\"newton_per_stage\": [",
                static_cast<long long>(m.ndof), static_cast<long long>(m.ne), m.colours.size(), m.col.size(),
                g_threads, setup_s, static_cast<long long>(nsteps), static_cast<long long>(r.newton),
                static_cast<long long>(r.timed_newton), r.seconds, r.asm_seconds, r.solve_seconds,
                static_cast<long long>(r.krylov), value, cpu_name().c_str(),
                g_precond == Precond::SSOR ? "SSOR" : "block Jacobi");
    for (size_t i = 0; i < r.newton_per_stage.size(); ++i)
      std::printf("%s%d", i ? ", " : "", r.newton_per_stage[i]);
    std::printf("]}\n");
  } catch (const std::exception& e) {
    std::fprintf(stderr, "cpu_newton: %s\n", e.what());
    std::printf("{\"error\": \"%s\"}\n", e.what());
    return 1;
  }
  return 0;
}
