// Math-expression front end: parser + compiler to register bytecode.
//
// Accepts the expression language of the reference's parser backends (default muParser,
// src/dune/copasi/parser/factory.cc:25-35; ExprTk, src/dune/copasi/parser/exprtk.cc) as
// documented in doc/docusaurus/docs/math_expr.mdx: muParser precedence (? : < || < && <
// comparisons < + - and prefix sign < * / % < ^ right-associative), 1/0 booleans,
// muParser and ExprTk built-in functions, parser_context constants, user functions of up
// to four arguments (src/dune/copasi/parser/context.cc:289-330), 1-D interpolation
// tables (context.cc:68-92), functions tabulated with `interpolate = true`
// (context.cc:237-280) and grayscale TIFF images (context.cc:62-67).
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
#include "lookup.hpp"
#include "tiff.hpp"

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

// a 1-argument function replaced by its values on a uniform grid (`interpolate = true`)
struct FnTable {
  FnTableDesc desc;           // desc.off = 0 here; set when the tables are packed
  std::vector<double> g;      // intervals + 1 values
};

class ParserContext {
 public:
  ParserContext() = default;
  explicit ParserContext(const Ini& cfg);
  std::map<std::string, double> constants;
  std::map<std::string, UserFunction> functions;
  std::map<std::string, int> tables;  // name -> index into interp
  std::vector<InterpTable> interp;
  std::map<std::string, int> fn_tables;  // name -> index into fn_table_data
  std::vector<FnTable> fn_table_data;
  std::map<std::string, int> images;     // name -> index into image_data (`tiff` entries)
  std::vector<TiffGray> image_data;
};

// host value of a table op (OP_INTERP, OP_FTAB, OP_TIFF) with table `index`
double eval_lookup(const ParserContext& ctx, uint8_t op, int index, double a, double c);

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
  // a parser-context function body: only its arguments (bound to nodes) and the
  // context-independent symbols (constants, interpolation tables, images) are visible
  int compile_function_body(const AstPtr& body, const std::map<std::string, int>& args);
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

// host evaluation of one op (constant folding and host-side checks); table ops go through
// eval_lookup
double eval_op(uint8_t op, double a, double b, double c, int8_t imm, const InterpTable* table);

// host evaluation of a compiled program (setup-time expressions: compartments, initial
// conditions, tabulated functions); inputs are given in the program's input order
double run_program_host(const Program& p, const ParserContext& ctx, const double* inputs,
                        int output = 0);

}  // namespace dcgpu
