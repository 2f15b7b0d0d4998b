// Math-expression front end: parser + compiler to register bytecode.
//
// Accepts the expression language of the reference's parser backends (default muParser,
// src/dune/copasi/parser/factory.cc:25-35; ExprTk, src/dune/copasi/parser/exprtk.cc) as
// documented in doc/docusaurus/docs/math_expr.mdx: muParser precedence (? : < || < && <
// comparisons < + - and prefix sign < * / % < ^ right-associative), 1/0 booleans,
// muParser and ExprTk built-in functions, parser_context constants, user functions of up
// to four arguments (src/dune/copasi/parser/context.cc:289-330) and 1-D interpolation
// tables (context.cc:68-92).
#pragma once

#include <functional>
#include <map>
#include <memory>
#include <optional>
#include <string>
#include <unordered_map>
#include <vector>

#include "bytecode.hpp"
#include "ini.hpp"

namespace dcgpu {

struct Ast {
  enum Kind { Num, Var, Neg, Not, Bin, Tern, Call } kind = Num;
  double num = 0.0;
  std::string name;  // Var / Call name, Bin operator
  std::vector<std::shared_ptr<Ast>> kids;
};
using AstPtr = std::shared_ptr<Ast>;

AstPtr parse_expression(const std::string& text);

// functor_factory_parser.impl.hh:121-128: an empty/all-zero expression means "no
// functor"; a bare float literal bypasses the parser.
bool is_zero_expression(const std::string& text);
std::optional<double> literal_value(const std::string& text);

struct UserFunction {
  std::vector<std::string> args;
  AstPtr body;
};

struct InterpTable {
  std::vector<double> x, y;
};

class ParserContext {
 public:
  ParserContext() = default;
  explicit ParserContext(const Ini& cfg);
  std::map<std::string, double> constants;
  std::map<std::string, UserFunction> functions;
  std::map<std::string, int> tables;  // name -> index into interp
  std::vector<InterpTable> interp;
};

// Value of a symbol: either a program input or a constant.
struct Symbol {
  bool is_input = false;
  uint16_t input = 0;
  double value = 0.0;
};
using Resolver = std::function<std::optional<Symbol>(const std::string&)>;

// Straight-line program over a register file (see bytecode.hpp).
struct Program {
  std::vector<Instr> code;
  std::vector<double> consts;
  std::vector<uint16_t> inputs;   // input i is loaded into register i
  std::vector<uint8_t> outputs;   // register holding output k
  int nregs = 0;
};

class ProgramBuilder {
 public:
  explicit ProgramBuilder(const ParserContext& ctx) : ctx_(ctx) {}
  // compile an expression; returns a node id
  int compile(const AstPtr& ast, const Resolver& resolve);
  int compile_text(const std::string& text, const Resolver& resolve);
  int constant(double v);
  int input(uint16_t id);
  int binary(uint8_t op, int a, int b);
  int unary(uint8_t op, int a);
  int add_output(int node);  // returns output index
  Program finish() const;
  bool is_constant(int node, double* v = nullptr) const;
  // true when the value of `node` reads an input whose id satisfies `pred`
  bool depends_on(int node, const std::function<bool(uint16_t)>& pred) const;

 private:
  struct Node {
    uint8_t op;  // OP_* ; 255 = input, 254 = constant
    int a = -1, b = -1, c = -1;
    double value = 0.0;
    uint16_t input = 0;
    int8_t imm = 0;
  };
  int intern(const Node& n);
  int fold_or_make(uint8_t op, int a, int b, int c, int8_t imm = 0);
  int compile_rec(const AstPtr& ast, const Resolver& resolve,
                  const std::map<std::string, int>* args);
  const ParserContext& ctx_;
  std::vector<Node> nodes_;
  std::unordered_map<std::string, int> memo_;
  std::vector<int> outputs_;
};

// host evaluation of one op (constant folding and host-side checks)
double eval_op(uint8_t op, double a, double b, double c, int8_t imm, const InterpTable* table);

}  // namespace dcgpu
