// Register bytecode for runtime math expressions, shared by the host compiler and the
// device interpreter.
//
// The reference evaluates every expression through a type-erased parser call per
// quadrature point (dune/copasi/model/functor_factory_parser.impl.hh:178-180 calling
// muParser / ExprTk / SymEngine, src/dune/copasi/parser/*.cc).  Here all expressions a
// kernel needs at one quadrature point are compiled into ONE straight-line program over
// a small register file: inputs are loaded into the first registers, common
// sub-expressions are shared, constants are folded, user functions are inlined, and the
// outputs are read back from registers.
#pragma once

#include <cstdint>

namespace dcgpu {

enum Op : uint8_t {
  OP_CONST = 0,  // r[dst] = consts[a | b<<8]
  OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_POW, OP_FMOD, OP_ATAN2, OP_HYPOT, OP_MIN, OP_MAX,
  OP_LT, OP_LE, OP_GT, OP_GE, OP_EQ, OP_NE, OP_AND, OP_OR,
  OP_NEG, OP_NOT, OP_SQR, OP_CUBE, OP_RECIP,
  OP_EXP, OP_LOG, OP_LOG2, OP_LOG10, OP_SQRT, OP_SIN, OP_COS, OP_TAN, OP_ASIN, OP_ACOS,
  OP_ATAN, OP_SINH, OP_COSH, OP_TANH, OP_ASINH, OP_ACOSH, OP_ATANH, OP_ABS, OP_SIGN,
  OP_RINT, OP_FLOOR, OP_CEIL, OP_ROUND, OP_TRUNC, OP_ERF, OP_ERFC,
  OP_SEL,      // r[dst] = r[a] != 0 ? r[b] : r[c]
  OP_POWI,     // r[dst] = r[a] ^ (int8)c   (small integer exponent, by multiplication)
  OP_INTERP,   // r[dst] = table[b](r[a])  (1-D linear interpolation, clamped)
  OP_FTAB,     // r[dst] = tabulated function b at r[a]  (`interpolate = true` functions)
  OP_TIFF,     // r[dst] = grayscale image b at (r[a], r[c])
  OP_COUNT
};

struct Instr {
  uint8_t op, dst, a, b, c, pad0, pad1, pad2;
};

// Symbols a program can read (the kernels fill the registers listed in the program's
// input table with these values).
enum InputKind : uint16_t {
  IN_SPECIES = 0,       // + species index (model-global)          -> value
  IN_GRAD = 1024,       // + species index * 3 + axis              -> gradient component
  IN_POSITION = 8192,   // + axis
  IN_NORMAL = 8200,     // + axis
  IN_TIME = 8300,
  IN_ENTITY_VOLUME,
  IN_IN_VOLUME,
  IN_IN_BOUNDARY,
  IN_IN_SKELETON,
  IN_INTEGRATION_FACTOR,
};

constexpr int kMaxRegisters = 64;
constexpr int kMaxInterpTables = 16;
constexpr int kMaxFnTables = 64;
constexpr int kMaxImages = 32;

}  // namespace dcgpu
