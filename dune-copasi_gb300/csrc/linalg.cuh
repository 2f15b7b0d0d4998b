// Sparse linear algebra on the device: BSR SpMV, fused Krylov vector updates with
// deterministic reductions, block-Jacobi preconditioning.
//
// Replaces the dune-istl operators the reference's LinearSolver drives
// (dune/copasi/model/make_step_operator.hh:102-146, solver/istl/factory/*.hh).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "sell.cuh"

namespace dcgpu {

struct Bsr {
  int nrows = 0;          // block rows
  int bs = 1;             // block size
  int64_t nnzb = 0;       // stored blocks
  const int32_t* rowptr = nullptr;
  const int32_t* colidx = nullptr;
  double* val = nullptr;  // nnzb * bs * bs, row-major blocks
  float* val32 = nullptr; // single-precision copy (mixed-precision Krylov)
};

// Reduction scratch: per-block partial sums and a completion counter.
struct ReduceScratch {
  double* partial = nullptr;    // kReduceBlocks * 4
  unsigned int* counter = nullptr;
  double* result = nullptr;     // device scalars written by the last block
};
constexpr int kReduceBlocks = 608;    // 4 x 152 SMs
constexpr int kReduceThreads = 256;

// y = A x   (fp64)
void spmv(const Bsr& A, const double* x, double* y, cudaStream_t s);
// y = A x   (fp32 values, fp32 vectors)
void spmv32(const Bsr& A, const float* x, float* y, cudaStream_t s);
// y = A x with the fp32 values `val` of A's pattern (thread per scalar row)
void spmv32_vals(const Bsr& A, const float* val, const float* x, float* y, cudaStream_t s);
// fp32 SELL-32 copy of the fp64 BSR values `val` (pattern of A, layout S); padding zeroed
void bsr_to_sell(const Bsr& A, const double* val, const Sell& S, float* out, cudaStream_t s);
// the same copy in fp64 (the batched fp64 Krylov solve reads the operator in this layout)
void bsr_to_sell64(const Bsr& A, const double* val, const Sell& S, double* out, cudaStream_t s);
// y = A x on the SELL-32 layout (warp per slice, lane per block row)
void spmv_sell32(const Sell& S, const float* val, const float* x, float* y, cudaStream_t s);
// r = b - A x (fp64)
void residual(const Bsr& A, const double* x, const double* b, double* r, cudaStream_t s);
// y += alpha * V x with the pattern of A and the values V (fp64)
void spmv_acc(const Bsr& A, const double* vals, const double* x, double* y, double alpha, cudaStream_t s);

// result[slot] = <x, y>  (deterministic; fixed grid and order)
void dot(const double* x, const double* y, int64_t n, ReduceScratch rs, int slot, cudaStream_t s);

// block Jacobi: dinv = inverse of the diagonal blocks; returns via status[0] != 0 on a
// singular block
// (dinv32, optional: the same inverses rounded to fp32)
void block_jacobi_setup(const Bsr& A, const int32_t* diag, double* dinv, int* status, cudaStream_t s,
                        float* dinv32 = nullptr);
void block_jacobi_apply(int nrows, int bs, const double* dinv, const double* x, double* y, cudaStream_t s);
void block_jacobi_apply32(int nrows, int bs, const float* dinv, const float* x, float* y, cudaStream_t s);

// number of kernels this library has launched (all threads, all models)
long long launch_count();
long long launch_count_this_thread();  // launches counted by the calling host thread
void count_launches(long long n);

// elementwise helpers
void axpy(int64_t n, double a, const double* x, double* y, cudaStream_t s);          // y += a x
void axpby(int64_t n, double a, const double* x, double b, double* y, cudaStream_t s); // y = a x + b y
void scale_copy(int64_t n, double a, const double* x, double* y, cudaStream_t s);     // y = a x
// out = a x + b y; x or y may be null (its term is left out)
void combine(int64_t n, double a, const double* x, double b, const double* y, double* out, cudaStream_t s);
void to_float(int64_t n, const double* x, float* y, cudaStream_t s);
// dst[idx[i]] = src[i] / dst[i] = src[idx[i]] for i < n (reference <-> blocked state layout)
void scatter_idx(int64_t n, const int64_t* idx, const double* src, double* dst, cudaStream_t s);
void gather_idx(int64_t n, const int64_t* idx, const double* src, double* dst, cudaStream_t s);
void add_float(int64_t n, const float* x, double* y, cudaStream_t s);                 // y += x
void to_float_scaled(int64_t n, const double* x, double scale, float* y, cudaStream_t s);
void add_float_scaled(int64_t n, const float* x, double scale, double* y, cudaStream_t s);
void fill(int64_t n, double v, double* y, cudaStream_t s);

}  // namespace dcgpu
