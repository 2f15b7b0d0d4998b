// Device interpreter for the expression bytecode (see bytecode.hpp), in FP64 (residuals,
// and every Jacobian outside the mixed-precision path) or FP32 (the Jacobian-only passes of
// the mixed-precision path, whose element matrices are rounded to FP32 anyway).  The FP32
// instantiation evaluates the same program with the single-precision math functions;
// table lookups stay in FP64.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "device.cuh"

namespace dcgpu {

__device__ __forceinline__ double interp_table(const DevTables& T, int tab, double x) {
  return interp_lookup(T.x + T.off[tab], T.y + T.off[tab], T.len[tab], x);
}

template <class F>
__device__ __forceinline__ F apply_op(const Instr ins, F a, F b, F c, const DevTables& T) {
  const F one = F(1), zero = F(0);
  switch (ins.op) {
    case OP_ADD: return a + b;
    case OP_SUB: return a - b;
    case OP_MUL: return a * b;
    case OP_DIV: return a / b;
    case OP_POW: return pow(a, b);
    case OP_FMOD: return fmod(a, b);
    case OP_ATAN2: return atan2(a, b);
    case OP_HYPOT: return hypot(a, b);
    case OP_MIN: return fmin(a, b);
    case OP_MAX: return fmax(a, b);
    case OP_LT: return a < b ? one : zero;
    case OP_LE: return a <= b ? one : zero;
    case OP_GT: return a > b ? one : zero;
    case OP_GE: return a >= b ? one : zero;
    case OP_EQ: return a == b ? one : zero;
    case OP_NE: return a != b ? one : zero;
    case OP_AND: return (a != zero && b != zero) ? one : zero;
    case OP_OR: return (a != zero || b != zero) ? one : zero;
    case OP_NEG: return -a;
    case OP_NOT: return a != zero ? zero : one;
    case OP_SQR: return a * a;
    case OP_CUBE: return a * a * a;
    case OP_RECIP: return one / a;
    case OP_EXP: return exp(a);
    case OP_LOG: return log(a);
    case OP_LOG2: return log2(a);
    case OP_LOG10: return log10(a);
    case OP_SQRT: return sqrt(a);
    case OP_SIN: return sin(a);
    case OP_COS: return cos(a);
    case OP_TAN: return tan(a);
    case OP_ASIN: return asin(a);
    case OP_ACOS: return acos(a);
    case OP_ATAN: return atan(a);
    case OP_SINH: return sinh(a);
    case OP_COSH: return cosh(a);
    case OP_TANH: return tanh(a);
    case OP_ASINH: return asinh(a);
    case OP_ACOSH: return acosh(a);
    case OP_ATANH: return atanh(a);
    case OP_ABS: return fabs(a);
    case OP_SIGN: return a < zero ? -one : (a > zero ? one : zero);
    case OP_RINT: return rint(a);
    case OP_FLOOR: return floor(a);
    case OP_CEIL: return ceil(a);
    case OP_ROUND: return round(a);
    case OP_TRUNC: return trunc(a);
    case OP_ERF: return erf(a);
    case OP_ERFC: return erfc(a);
    case OP_SEL: return a != zero ? b : c;
    case OP_POWI: {
      int e = static_cast<int8_t>(ins.c);
      int n = e < 0 ? -e : e;
      F r = one, x = a;
      while (n) {
        if (n & 1) r *= x;
        x *= x;
        n >>= 1;
      }
      return e < 0 ? one / r : r;
    }
    case OP_INTERP: return static_cast<F>(interp_table(T, ins.b, static_cast<double>(a)));
    case OP_FTAB: return static_cast<F>(ftab_lookup(T.ft[ins.b], T.ftg, static_cast<double>(a)));
    case OP_TIFF:
      return static_cast<F>(image_lookup(T.im[ins.b], T.imp, static_cast<double>(a), static_cast<double>(c)));
    default: return static_cast<F>(__longlong_as_double(0x7ff8000000000000ULL));
  }
}

// Run a program; inputs must already be in R[0..ninputs).  All threads of a warp run the
// same instruction stream, so the dispatch is uniform.
template <class F, class Regs>
__device__ __forceinline__ void run_program(const DevProgram& P, const DevTables& T, Regs R) {
  for (int pc = 0; pc < P.ncode; ++pc) {
    const Instr ins = P.code[pc];
    F v;
    if (ins.op == OP_CONST) {
      // FP32 programs read the constants pre-rounded: a double-to-float conversion per use
      // runs on the FP64 pipe
      if constexpr (std::is_same_v<F, float>) v = P.consts32[ins.a | (ins.b << 8)];
      else v = P.consts[ins.a | (ins.b << 8)];
    } else {
      const F a = R[ins.a];
      const bool table = ins.op == OP_INTERP || ins.op == OP_FTAB || ins.op == OP_TIFF;
      const F b = (ins.op == OP_POWI || table) ? F(0) : R[ins.b];
      const F c = (ins.op == OP_SEL || ins.op == OP_TIFF) ? R[ins.c] : F(0);
      v = apply_op<F>(ins, a, b, c, T);
    }
    R[ins.dst] = v;
  }
}

}  // namespace dcgpu
