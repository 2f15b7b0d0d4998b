#include "expr.hpp"

#include <cctype>
#include <cmath>
#include <cstring>
#include <regex>
#include <set>
#include <sstream>

namespace dcgpu {

// ------------------------------------------------------------------ tokenizer / parser

namespace {

struct Tok {
  enum Kind { End, Num, Id, Op } kind = End;
  double num = 0.0;
  std::string s;
};

std::vector<Tok> tokenize(const std::string& text) {
  std::vector<Tok> out;
  size_t i = 0, n = text.size();
  while (i < n) {
    unsigned char ch = static_cast<unsigned char>(text[i]);
    if (std::isspace(ch)) { ++i; continue; }
    if (std::isdigit(ch) || (ch == '.' && i + 1 < n && std::isdigit(static_cast<unsigned char>(text[i + 1])))) {
      size_t j = i;
      while (j < n && std::isdigit(static_cast<unsigned char>(text[j]))) ++j;
      if (j < n && text[j] == '.') { ++j; while (j < n && std::isdigit(static_cast<unsigned char>(text[j]))) ++j; }
      if (j < n && (text[j] == 'e' || text[j] == 'E')) {
        size_t k = j + 1;
        if (k < n && (text[k] == '+' || text[k] == '-')) ++k;
        if (k < n && std::isdigit(static_cast<unsigned char>(text[k]))) {
          j = k;
          while (j < n && std::isdigit(static_cast<unsigned char>(text[j]))) ++j;
        }
      }
      Tok t; t.kind = Tok::Num; t.num = std::strtod(text.substr(i, j - i).c_str(), nullptr);
      out.push_back(t); i = j; continue;
    }
    if (std::isalpha(ch) || ch == '_') {
      size_t j = i;
      while (j < n && (std::isalnum(static_cast<unsigned char>(text[j])) || text[j] == '_')) ++j;
      Tok t; t.kind = Tok::Id; t.s = text.substr(i, j - i);
      out.push_back(t); i = j; continue;
    }
    static const char* two[] = {"||", "&&", "==", "!=", "<>", "<=", ">="};
    bool matched = false;
    for (const char* op : two) {
      if (text.compare(i, 2, op) == 0) {
        Tok t; t.kind = Tok::Op; t.s = op; out.push_back(t); i += 2; matched = true; break;
      }
    }
    if (matched) continue;
    if (std::strchr("-+*/%^<>=!?:(),", ch)) {
      Tok t; t.kind = Tok::Op; t.s = std::string(1, static_cast<char>(ch)); out.push_back(t); ++i; continue;
    }
    throw ConfigError("unexpected character '" + std::string(1, static_cast<char>(ch)) + "' in expression '" + text + "'");
  }
  out.push_back(Tok{});
  return out;
}

int binary_precedence(const Tok& t, std::string* canon) {
  static const std::map<std::string, int> prec = {
      {"||", 1}, {"or", 1}, {"&&", 2}, {"and", 2}, {"==", 5}, {"=", 5}, {"!=", 5}, {"<>", 5},
      {"<", 5},  {"<=", 5}, {">", 5},  {">=", 5},  {"+", 6},  {"-", 6}, {"*", 7},  {"/", 7},
      {"%", 7},  {"^", 8}};
  if (t.kind != Tok::Op && !(t.kind == Tok::Id && (t.s == "and" || t.s == "or"))) return -1;
  auto it = prec.find(t.s);
  if (it == prec.end()) return -1;
  if (canon) {
    if (t.s == "or") *canon = "||";
    else if (t.s == "and") *canon = "&&";
    else if (t.s == "=") *canon = "==";
    else if (t.s == "<>") *canon = "!=";
    else *canon = t.s;
  }
  return it->second;
}

class AstParser {
 public:
  explicit AstParser(const std::string& text) : text_(text), toks_(tokenize(text)) {}
  AstPtr parse() {
    auto n = ternary();
    if (peek().kind != Tok::End) fail("trailing input");
    return n;
  }

 private:
  const Tok& peek() const { return toks_[i_]; }
  Tok take() { return toks_[i_++]; }
  bool is_op(const char* s) const { return peek().kind == Tok::Op && peek().s == s; }
  [[noreturn]] void fail(const std::string& what) const {
    throw ConfigError(what + " in expression '" + text_ + "'");
  }
  void expect(const char* s) {
    if (!is_op(s)) fail(std::string("expected '") + s + "'");
    take();
  }
  static AstPtr make(Ast::Kind k) { auto a = std::make_shared<Ast>(); a->kind = k; return a; }

  AstPtr ternary() {
    auto c = binary(1);
    if (is_op("?")) {
      take();
      auto a = ternary();
      expect(":");
      auto b = ternary();
      auto t = make(Ast::Tern);
      t->kids = {c, a, b};
      return t;
    }
    return c;
  }
  AstPtr binary(int min_prec) {
    auto lhs = unary();
    while (true) {
      std::string op;
      int p = binary_precedence(peek(), &op);
      if (p < 0 || p < min_prec) return lhs;
      take();
      AstPtr rhs = (op == "^") ? binary(8) : binary(p + 1);
      auto b = make(Ast::Bin);
      b->name = op;
      b->kids = {lhs, rhs};
      lhs = b;
    }
  }
  AstPtr unary() {
    if (is_op("-")) { take(); auto n = make(Ast::Neg); n->kids = {binary(7)}; return n; }
    if (is_op("+")) { take(); return binary(7); }
    if (is_op("!") || (peek().kind == Tok::Id && peek().s == "not")) {
      take(); auto n = make(Ast::Not); n->kids = {binary(7)}; return n;
    }
    return primary();
  }
  AstPtr primary() {
    Tok t = take();
    if (t.kind == Tok::Num) { auto n = make(Ast::Num); n->num = t.num; return n; }
    if (t.kind == Tok::Op && t.s == "(") { auto n = ternary(); expect(")"); return n; }
    if (t.kind == Tok::Id) {
      if (is_op("(")) {
        take();
        auto c = make(Ast::Call);
        c->name = t.s;
        if (!is_op(")")) {
          c->kids.push_back(ternary());
          while (is_op(",")) { take(); c->kids.push_back(ternary()); }
        }
        expect(")");
        return c;
      }
      auto v = make(Ast::Var);
      v->name = t.s;
      return v;
    }
    fail("unexpected token '" + t.s + "'");
  }

  std::string text_;
  std::vector<Tok> toks_;
  size_t i_ = 0;
};

}  // namespace

AstPtr parse_expression(const std::string& text) { return AstParser(text).parse(); }

bool is_zero_expression(const std::string& text) {
  static const std::regex zero_re("-?([0]+)?([\\.]?)([0]+)?");
  return text.empty() || std::regex_match(text, zero_re);
}

std::optional<double> literal_value(const std::string& text) {
  static const std::regex float_re("-?([0-9]+)?([\\.]?)([0-9]+)?");
  if (std::regex_match(text, float_re)) return std::strtod(text.c_str(), nullptr);
  return std::nullopt;
}

// ------------------------------------------------------------------ parser context

ParserContext::ParserContext(const Ini& cfg) {
  std::vector<std::pair<std::string, Ini>> tabulate;  // `interpolate = true` functions
  for (const auto& name : cfg.sub_keys()) {
    Ini sub = cfg.sub(name);
    std::string type = sub.get("type", "");
    if (type == "constant") {
      constants[name] = sub.get_double("value", 0.0);
    } else if (type == "tiff") {
      if (static_cast<int>(image_data.size()) >= kMaxImages) throw ConfigError("too many tiff images");
      images[name] = static_cast<int>(image_data.size());
      image_data.push_back(read_tiff_gray(sub.at("path")));
    } else if (type == "random_field") {
      // context.cc:93-160 needs the optional parafields library; a reference build without
      // it rejects the type with this message
      throw ConfigError("Library was compiled without random fields support");
    } else if (type == "cell_data") {
      throw ConfigError("cell data is not implemented");  // context.cc:161-162
    } else if (type == "function") {
      if (sub.get_bool("interpolate", false)) {
        tabulate.emplace_back(name, sub);
        continue;
      }
      std::string e = sub.at("expression");
      auto colon = e.find(':');
      if (colon == std::string::npos)
        throw ConfigError("function '" + name + "' needs the form 'args: expression'");
      UserFunction f;
      std::string head = e.substr(0, colon);
      std::stringstream ss(head);
      std::string a;
      while (std::getline(ss, a, ',')) {
        a = trim(a);
        if (!a.empty()) f.args.push_back(a);
      }
      if (f.args.size() > 4) throw ConfigError("function '" + name + "' has more than 4 arguments");
      f.body = parse_expression(e.substr(colon + 1));
      functions[name] = f;
    } else if (type == "interpolation") {
      InterpTable t;
      t.x = sub.get_doubles("domain", {});
      t.y = sub.get_doubles("range", {});
      for (size_t k = 1; k < t.x.size(); ++k)
        if (t.x[k] < t.x[k - 1]) throw ConfigError("The interpolation domain must be sorted");
      if (t.x.size() < 2 || t.x.size() != t.y.size())
        throw ConfigError("Interpolation range and domain must have at least two points and be the same size");
      if (static_cast<int>(interp.size()) >= kMaxInterpTables) throw ConfigError("too many interpolation tables");
      tables[name] = static_cast<int>(interp.size());
      interp.push_back(t);
    } else {
      throw ConfigError("Unknown type " + type);
    }
  }

  // context.cc:237-280: a 1-argument function evaluated on intervals + 1 points of its
  // domain and replaced by a lookup into those values.  The bodies see the constants,
  // interpolation tables and images, not other expression functions (tables made here are
  // registered only after all of them are built).
  std::vector<std::pair<std::string, FnTable>> made;
  for (const auto& [name, sub] : tabulate) {
    std::string e = sub.at("expression");
    auto colon = e.find(':');
    if (colon == std::string::npos) throw ConfigError("Function arguments must precede a colon ':'");
    std::vector<std::string> args;
    std::stringstream ss(e.substr(0, colon));
    for (std::string a; std::getline(ss, a, ',');)
      if (!trim(a).empty()) args.push_back(trim(a));
    if (args.size() != 1)
      throw ConfigError("Cannot interpolate '" + name + "' function with " + std::to_string(args.size()) +
                        " arguments");
    const long intervals = sub.get_long("interpolation.intervals", 1000);
    if (intervals > 100000) throw ConfigError("Number of interpolation intervals is too big!");
    if (intervals < 1) throw ConfigError("At least one interval is required in function " + name);
    const auto dom = sub.get_doubles("interpolation.domain." + args[0], {0.0, 1.0});
    if (dom.size() != 2) throw ConfigError("interpolation.domain." + args[0] + " needs two values");
    if (dom[0] >= dom[1]) {
      std::ostringstream m;
      m << "Domain arguments (" << dom[0] << ", " << dom[1] << ") of function " << name << " are not ordered";
      throw ConfigError(m.str());
    }
    const std::string ooo = sub.get("interpolation.out_of_bounds", "error");
    if (ooo != "clamp" && ooo != "error")
      throw ConfigError("Not known '" + name + ".interpolation.out_of_bounds = " + ooo + "'");
    ProgramBuilder pb(*this);
    std::map<std::string, int> bound{{args[0], pb.input(0)}};
    pb.add_output(pb.compile_function_body(parse_expression(e.substr(colon + 1)), bound));
    const Program p = pb.finish();
    FnTable t;
    t.desc.d0 = dom[0];
    t.desc.d1 = dom[1];
    t.desc.intervals = static_cast<uint32_t>(intervals);
    t.desc.clamp = ooo == "clamp" ? 1 : 0;
    const double nf = static_cast<double>(intervals);
    const double width = (dom[1] - dom[0]) / nf;
    t.desc.ctn = nf / (dom[1] - dom[0]);
    t.g.resize(static_cast<size_t>(intervals) + 1);
    for (size_t i = 0; i < t.g.size(); ++i) {
      const double x = dom[0] + static_cast<double>(i) * width;
      t.g[i] = run_program_host(p, *this, &x);
    }
    made.emplace_back(name, std::move(t));
  }
  for (auto& [name, t] : made) {
    if (static_cast<int>(fn_table_data.size()) >= kMaxFnTables) throw ConfigError("too many tabulated functions");
    fn_tables[name] = static_cast<int>(fn_table_data.size());
    fn_table_data.push_back(std::move(t));
  }
}

double run_program_host(const Program& p, const ParserContext& ctx, const double* inputs, int output) {
  std::vector<double> R(std::max(p.nregs, 1), 0.0);
  for (size_t i = 0; i < p.inputs.size(); ++i) R[i] = inputs[i];
  for (const Instr& ins : p.code) {
    if (ins.op == OP_CONST) {
      R[ins.dst] = p.consts[ins.a | (ins.b << 8)];
    } else if (ins.op == OP_INTERP || ins.op == OP_FTAB || ins.op == OP_TIFF) {
      R[ins.dst] = eval_lookup(ctx, ins.op, ins.b, R[ins.a], R[ins.c]);
    } else {
      R[ins.dst] = eval_op(ins.op, R[ins.a], R[ins.b], R[ins.c], static_cast<int8_t>(ins.c), nullptr);
    }
  }
  return R[p.outputs.at(output)];
}

double eval_lookup(const ParserContext& ctx, uint8_t op, int index, double a, double c) {
  switch (op) {
    case OP_INTERP: {
      const InterpTable& t = ctx.interp.at(index);
      return interp_lookup(t.x.data(), t.y.data(), static_cast<int>(t.x.size()), a);
    }
    case OP_FTAB: {
      const FnTable& t = ctx.fn_table_data.at(index);
      FnTableDesc d = t.desc;
      d.off = 0;
      return ftab_lookup(d, t.g.data(), a);
    }
    case OP_TIFF: {
      const TiffGray& im = ctx.image_data.at(index);
      ImageDesc d;
      d.rows = im.rows;
      d.cols = im.cols;
      d.x_res = im.x_res;
      d.y_res = im.y_res;
      d.x_off = im.x_off;
      d.y_off = im.y_off;
      return image_lookup(d, im.px.data(), a, c);
    }
    default: return std::nan("");
  }
}

// ------------------------------------------------------------------ evaluation (host)

double eval_op(uint8_t op, double a, double b, double c, int8_t imm, const InterpTable* table) {
  switch (op) {
    case OP_ADD: return a + b;
    case OP_SUB: return a - b;
    case OP_MUL: return a * b;
    case OP_DIV: return a / b;
    case OP_POW: return std::pow(a, b);
    case OP_FMOD: return std::fmod(a, b);
    case OP_ATAN2: return std::atan2(a, b);
    case OP_HYPOT: return std::hypot(a, b);
    case OP_MIN: return std::fmin(a, b);
    case OP_MAX: return std::fmax(a, b);
    case OP_LT: return a < b ? 1.0 : 0.0;
    case OP_LE: return a <= b ? 1.0 : 0.0;
    case OP_GT: return a > b ? 1.0 : 0.0;
    case OP_GE: return a >= b ? 1.0 : 0.0;
    case OP_EQ: return a == b ? 1.0 : 0.0;
    case OP_NE: return a != b ? 1.0 : 0.0;
    case OP_AND: return (a != 0.0 && b != 0.0) ? 1.0 : 0.0;
    case OP_OR: return (a != 0.0 || b != 0.0) ? 1.0 : 0.0;
    case OP_NEG: return -a;
    case OP_NOT: return a != 0.0 ? 0.0 : 1.0;
    case OP_SQR: return a * a;
    case OP_CUBE: return a * a * a;
    case OP_RECIP: return 1.0 / a;
    case OP_EXP: return std::exp(a);
    case OP_LOG: return std::log(a);
    case OP_LOG2: return std::log2(a);
    case OP_LOG10: return std::log10(a);
    case OP_SQRT: return std::sqrt(a);
    case OP_SIN: return std::sin(a);
    case OP_COS: return std::cos(a);
    case OP_TAN: return std::tan(a);
    case OP_ASIN: return std::asin(a);
    case OP_ACOS: return std::acos(a);
    case OP_ATAN: return std::atan(a);
    case OP_SINH: return std::sinh(a);
    case OP_COSH: return std::cosh(a);
    case OP_TANH: return std::tanh(a);
    case OP_ASINH: return std::asinh(a);
    case OP_ACOSH: return std::acosh(a);
    case OP_ATANH: return std::atanh(a);
    case OP_ABS: return std::fabs(a);
    case OP_SIGN: return a < 0.0 ? -1.0 : (a > 0.0 ? 1.0 : 0.0);
    case OP_RINT: return std::rint(a);
    case OP_FLOOR: return std::floor(a);
    case OP_CEIL: return std::ceil(a);
    case OP_ROUND: return std::round(a);
    case OP_TRUNC: return std::trunc(a);
    case OP_ERF: return std::erf(a);
    case OP_ERFC: return std::erfc(a);
    case OP_SEL: return a != 0.0 ? b : c;
    case OP_POWI: {
      int n = imm < 0 ? -imm : imm;
      double r = 1.0, x = a;
      while (n) { if (n & 1) r *= x; x *= x; n >>= 1; }
      return imm < 0 ? 1.0 / r : r;
    }
    case OP_INTERP:
      if (!table) return std::nan("");
      return interp_lookup(table->x.data(), table->y.data(), static_cast<int>(table->x.size()), a);
    default: return std::nan("");
  }
}

// ------------------------------------------------------------------ program builder

int ProgramBuilder::intern(const Node& n) {
  std::ostringstream key;
  key << int(n.op) << ':' << n.a << ':' << n.b << ':' << n.c << ':' << int(n.imm) << ':' << n.input << ':';
  if (n.op == 254) {
    uint64_t bits;
    std::memcpy(&bits, &n.value, sizeof bits);
    key << bits;
  }
  auto k = key.str();
  auto it = memo_.find(k);
  if (it != memo_.end()) return it->second;
  nodes_.push_back(n);
  int id = static_cast<int>(nodes_.size()) - 1;
  memo_[k] = id;
  return id;
}

int ProgramBuilder::constant(double v) {
  Node n; n.op = 254; n.value = v;
  return intern(n);
}

int ProgramBuilder::input(uint16_t id) {
  Node n; n.op = 255; n.input = id;
  return intern(n);
}

bool ProgramBuilder::is_constant(int node, double* v) const {
  if (nodes_[node].op != 254) return false;
  if (v) *v = nodes_[node].value;
  return true;
}

bool ProgramBuilder::depends_on(int node, const std::function<bool(uint16_t)>& pred) const {
  std::vector<int> stack{node};
  std::vector<char> seen(nodes_.size(), 0);
  while (!stack.empty()) {
    int k = stack.back();
    stack.pop_back();
    if (k < 0 || seen[k]) continue;
    seen[k] = 1;
    const Node& n = nodes_[k];
    if (n.op == 255 && pred(n.input)) return true;
    stack.push_back(n.a);
    stack.push_back(n.b);
    stack.push_back(n.c);
  }
  return false;
}

int ProgramBuilder::fold_or_make(uint8_t op, int a, int b, int c, int8_t imm) {
  double va = 0, vb = 0, vc = 0;
  bool ca = a < 0 || is_constant(a, &va);
  bool cb = b < 0 || is_constant(b, &vb);
  bool cc = c < 0 || is_constant(c, &vc);
  if (ca && cb && cc && op != OP_INTERP) return constant(eval_op(op, va, vb, vc, imm, nullptr));
  if (op == OP_SEL && is_constant(a, &va)) return va != 0.0 ? b : c;
  // identities that hold bit for bit in IEEE arithmetic (x * 1, 1 * x, x / 1, x - 0 are x
  // for every x, signed zeros, infinities and NaN included)
  if (op == OP_MUL && ca && va == 1.0) return b;
  if ((op == OP_MUL || op == OP_DIV) && cb && vb == 1.0) return a;
  if (op == OP_SUB && cb && vb == 0.0 && !std::signbit(vb)) return a;
  Node n; n.op = op; n.a = a; n.b = b; n.c = c; n.imm = imm;
  return intern(n);
}

int ProgramBuilder::binary(uint8_t op, int a, int b) {
  double vb;
  if (op == OP_POW && is_constant(b, &vb) && vb == std::floor(vb) && std::fabs(vb) <= 16.0) {
    int e = static_cast<int>(vb);
    if (e == 1) return a;
    if (e == 2) return fold_or_make(OP_SQR, a, -1, -1);
    if (e == 3) return fold_or_make(OP_CUBE, a, -1, -1);
    if (e == -1) return fold_or_make(OP_RECIP, a, -1, -1);
    if (e == 0) return constant(1.0);
    return fold_or_make(OP_POWI, a, -1, -1, static_cast<int8_t>(e));
  }
  return fold_or_make(op, a, b, -1);
}

int ProgramBuilder::unary(uint8_t op, int a) { return fold_or_make(op, a, -1, -1); }

int ProgramBuilder::compile_text(const std::string& text, const Resolver& resolve) {
  if (auto v = literal_value(trim(text))) return constant(*v);
  return compile(parse_expression(text), resolve);
}

int ProgramBuilder::compile(const AstPtr& ast, const Resolver& resolve) {
  return compile_rec(ast, resolve, nullptr);
}

int ProgramBuilder::compile_function_body(const AstPtr& body, const std::map<std::string, int>& args) {
  Resolver none = [](const std::string&) -> std::optional<Symbol> { return std::nullopt; };
  return compile_rec(body, none, &args);
}

int ProgramBuilder::compile_rec(const AstPtr& ast, const Resolver& resolve,
                                const std::map<std::string, int>* args) {
  switch (ast->kind) {
    case Ast::Num: return constant(ast->num);
    case Ast::Var: {
      const std::string& nm = ast->name;
      if (args) {
        auto it = args->find(nm);
        if (it != args->end()) return it->second;
      }
      if (auto s = resolve(nm)) return s->is_input ? input(s->input) : constant(s->value);
      auto c = ctx_.constants.find(nm);
      if (c != ctx_.constants.end()) return constant(c->second);
      if (nm == "_pi") return constant(M_PI);
      if (nm == "_e") return constant(M_E);
      if (nm == "true") return constant(1.0);
      if (nm == "false") return constant(0.0);
      throw ConfigError("unknown symbol '" + nm + "'");
    }
    case Ast::Neg: return unary(OP_NEG, compile_rec(ast->kids[0], resolve, args));
    case Ast::Not: return unary(OP_NOT, compile_rec(ast->kids[0], resolve, args));
    case Ast::Tern: {
      int c = compile_rec(ast->kids[0], resolve, args);
      int a = compile_rec(ast->kids[1], resolve, args);
      int b = compile_rec(ast->kids[2], resolve, args);
      return fold_or_make(OP_SEL, c, a, b);
    }
    case Ast::Bin: {
      static const std::map<std::string, uint8_t> ops = {
          {"+", OP_ADD}, {"-", OP_SUB}, {"*", OP_MUL}, {"/", OP_DIV}, {"%", OP_FMOD},
          {"^", OP_POW}, {"<", OP_LT},  {"<=", OP_LE}, {">", OP_GT},  {">=", OP_GE},
          {"==", OP_EQ}, {"!=", OP_NE}, {"&&", OP_AND}, {"||", OP_OR}};
      int a = compile_rec(ast->kids[0], resolve, args);
      int b = compile_rec(ast->kids[1], resolve, args);
      return binary(ops.at(ast->name), a, b);
    }
    case Ast::Call: {
      const std::string& f = ast->name;
      std::vector<int> a;
      for (const auto& k : ast->kids) a.push_back(compile_rec(k, resolve, args));
      auto uf = ctx_.functions.find(f);
      if (uf != ctx_.functions.end()) {
        if (args) throw ConfigError("user function '" + f + "' may not call other user functions");
        if (a.size() != uf->second.args.size())
          throw ConfigError("function '" + f + "' takes " + std::to_string(uf->second.args.size()) + " arguments");
        std::map<std::string, int> bound;
        for (size_t k = 0; k < a.size(); ++k) bound[uf->second.args[k]] = a[k];
        // the body sees its arguments and the context constants only
        Resolver none = [](const std::string&) -> std::optional<Symbol> { return std::nullopt; };
        return compile_rec(uf->second.body, none, &bound);
      }
      auto tb = ctx_.tables.find(f);
      if (tb != ctx_.tables.end()) {
        if (a.size() != 1) throw ConfigError("interpolation '" + f + "' takes one argument");
        double v;
        if (is_constant(a[0], &v)) return constant(eval_op(OP_INTERP, v, 0, 0, 0, &ctx_.interp[tb->second]));
        Node n; n.op = OP_INTERP; n.a = a[0]; n.imm = static_cast<int8_t>(tb->second);
        return intern(n);
      }
      // functions tabulated with `interpolate = true`: expression functions, so a body may
      // not call them either
      auto ft = ctx_.fn_tables.find(f);
      if (ft != ctx_.fn_tables.end()) {
        if (args) throw ConfigError("user function '" + f + "' may not call other user functions");
        if (a.size() != 1) throw ConfigError("function '" + f + "' takes 1 arguments");
        double v;
        if (is_constant(a[0], &v)) return constant(eval_lookup(ctx_, OP_FTAB, ft->second, v, 0.0));
        Node n; n.op = OP_FTAB; n.a = a[0]; n.imm = static_cast<int8_t>(ft->second);
        return intern(n);
      }
      // grayscale images: f(x, y)
      auto im = ctx_.images.find(f);
      if (im != ctx_.images.end()) {
        if (a.size() != 2) throw ConfigError("tiff function '" + f + "' takes two arguments");
        double vx, vy;
        if (is_constant(a[0], &vx) && is_constant(a[1], &vy))
          return constant(eval_lookup(ctx_, OP_TIFF, im->second, vx, vy));
        Node n; n.op = OP_TIFF; n.a = a[0]; n.c = a[1]; n.imm = static_cast<int8_t>(im->second);
        return intern(n);
      }
      static const std::map<std::string, uint8_t> un = {
          {"exp", OP_EXP},     {"log", OP_LOG},     {"ln", OP_LOG},       {"log2", OP_LOG2},
          {"log10", OP_LOG10}, {"sqrt", OP_SQRT},   {"sin", OP_SIN},      {"cos", OP_COS},
          {"tan", OP_TAN},     {"asin", OP_ASIN},   {"acos", OP_ACOS},    {"atan", OP_ATAN},
          {"sinh", OP_SINH},   {"cosh", OP_COSH},   {"tanh", OP_TANH},    {"asinh", OP_ASINH},
          {"acosh", OP_ACOSH}, {"atanh", OP_ATANH}, {"abs", OP_ABS},      {"sign", OP_SIGN},
          {"rint", OP_RINT},   {"floor", OP_FLOOR}, {"ceil", OP_CEIL},    {"round", OP_ROUND},
          {"trunc", OP_TRUNC}, {"erf", OP_ERF},     {"erfc", OP_ERFC}};
      auto check = [&](size_t lo, size_t hi) {
        if (a.size() < lo || a.size() > hi) throw ConfigError("wrong number of arguments for '" + f + "'");
      };
      auto u = un.find(f);
      if (u != un.end()) { check(1, 1); return unary(u->second, a[0]); }
      if (f == "pow") { check(2, 2); return binary(OP_POW, a[0], a[1]); }
      if (f == "atan2") { check(2, 2); return binary(OP_ATAN2, a[0], a[1]); }
      if (f == "hypot") { check(2, 2); return binary(OP_HYPOT, a[0], a[1]); }
      if (f == "if") { check(3, 3); return fold_or_make(OP_SEL, a[0], a[1], a[2]); }
      if (f == "clamp") { check(3, 3); return binary(OP_MIN, binary(OP_MAX, a[1], a[0]), a[2]); }
      if (f == "min" || f == "max" || f == "sum" || f == "avg") {
        check(1, 64);
        uint8_t op = f == "min" ? OP_MIN : f == "max" ? OP_MAX : OP_ADD;
        int r = a[0];
        for (size_t k = 1; k < a.size(); ++k) r = binary(op, r, a[k]);
        if (f == "avg") r = binary(OP_DIV, r, constant(static_cast<double>(a.size())));
        return r;
      }
      throw ConfigError("unknown function '" + f + "'");
    }
  }
  throw ConfigError("bad expression node");
}

int ProgramBuilder::add_output(int node) {
  outputs_.push_back(node);
  return static_cast<int>(outputs_.size()) - 1;
}

Program ProgramBuilder::finish() const {
  Program p;
  // Divisions that share a non-constant divisor (Vmax*s/(Km+s) next to its derivative
  // Vmax*Km/(Km+s)^2 ...) take one reciprocal and multiply: a FP64 division costs a
  // reciprocal plus refinement, a multiplication one FMA-pipe instruction.  a*(1/d) is
  // within 1.5 ulp of a/d.
  std::vector<int> div_uses(nodes_.size(), 0);
  for (const Node& nd : nodes_)
    if (nd.op == OP_DIV && nd.b >= 0 && !is_constant(nd.b, nullptr)) ++div_uses[nd.b];
  std::vector<Node> nodes;
  nodes.reserve(nodes_.size() + 8);
  std::vector<int> remap(nodes_.size(), -1), rcp_of(nodes_.size(), -1);
  auto mapped = [&](int k) { return k >= 0 ? remap[k] : -1; };
  for (size_t i = 0; i < nodes_.size(); ++i) {
    Node nd = nodes_[i];
    if (nd.op == OP_DIV && nd.b >= 0 && div_uses[nd.b] >= 2) {
      if (rcp_of[nd.b] < 0) {
        Node r;
        r.op = OP_RECIP;
        r.a = remap[nd.b];
        r.b = -1;
        r.c = -1;
        nodes.push_back(r);
        rcp_of[nd.b] = static_cast<int>(nodes.size()) - 1;
      }
      Node m;
      m.op = OP_MUL;
      m.a = remap[nd.a];
      m.b = rcp_of[nd.b];
      m.c = -1;
      nodes.push_back(m);
    } else {
      nd.a = mapped(nd.a);
      nd.b = mapped(nd.b);
      nd.c = mapped(nd.c);
      nodes.push_back(nd);
    }
    remap[i] = static_cast<int>(nodes.size()) - 1;
  }
  std::vector<int> outputs;
  for (int o : outputs_) outputs.push_back(remap[o]);
  const int n = static_cast<int>(nodes.size());
  // live range ends
  std::vector<int> last(n, -1);
  for (int i = 0; i < n; ++i) {
    const Node& nd = nodes[i];
    for (int k : {nd.a, nd.b, nd.c})
      if (k >= 0) last[k] = std::max(last[k], i);
  }
  for (int o : outputs) last[o] = n;  // outputs stay live to the end
  // reachable nodes only
  std::vector<char> need(n, 0);
  for (int o : outputs) need[o] = 1;
  for (int i = n - 1; i >= 0; --i) {
    if (!need[i]) continue;
    const Node& nd = nodes[i];
    for (int k : {nd.a, nd.b, nd.c})
      if (k >= 0) need[k] = 1;
  }
  std::vector<int> reg(n, -1);
  std::vector<int> free_regs;
  int nregs = 0;
  // inputs first, in registers 0..
  for (int i = 0; i < n; ++i) {
    if (need[i] && nodes[i].op == 255) {
      reg[i] = nregs++;
      p.inputs.push_back(nodes[i].input);
    }
  }
  // simple linear scan: expire operands whose last use is this node
  std::vector<std::vector<int>> expire(n + 1);
  for (int i = 0; i < n; ++i)
    if (need[i] && last[i] >= 0 && last[i] < n) expire[last[i]].push_back(i);
  for (int i = 0; i < n; ++i) {
    if (!need[i]) continue;
    const Node& nd = nodes[i];
    if (nd.op == 255) continue;
    // operands that die here can give their register to the result
    for (int k : expire[i])
      if (reg[k] >= 0) free_regs.push_back(reg[k]);
    int r;
    if (!free_regs.empty()) { r = free_regs.back(); free_regs.pop_back(); }
    else r = nregs++;
    reg[i] = r;
    if (nregs > kMaxRegisters) throw ConfigError("expression program needs too many registers");
    Instr ins{};
    ins.dst = static_cast<uint8_t>(r);
    if (nd.op == 254) {
      int idx = static_cast<int>(p.consts.size());
      p.consts.push_back(nd.value);
      ins.op = OP_CONST;
      ins.a = static_cast<uint8_t>(idx & 0xff);
      ins.b = static_cast<uint8_t>((idx >> 8) & 0xff);
    } else {
      ins.op = nd.op;
      ins.a = nd.a >= 0 ? static_cast<uint8_t>(reg[nd.a]) : 0;
      ins.b = nd.b >= 0 ? static_cast<uint8_t>(reg[nd.b]) : 0;
      ins.c = nd.c >= 0 ? static_cast<uint8_t>(reg[nd.c]) : 0;
      if (nd.op == OP_POWI) ins.c = static_cast<uint8_t>(nd.imm);
      if (nd.op == OP_INTERP || nd.op == OP_FTAB || nd.op == OP_TIFF) ins.b = static_cast<uint8_t>(nd.imm);
    }
    p.code.push_back(ins);
  }
  for (int o : outputs) p.outputs.push_back(static_cast<uint8_t>(reg[o]));
  p.nregs = nregs;
  return p;
}

}  // namespace dcgpu
