// Block-Jacobi preconditioned BiCGSTAB with device-side convergence control.
//
// Replaces the dune-istl BiCGSTABSolver that the reference's LinearSolver drives
// (dune/copasi/model/make_step_operator.hh:102-146, solver/istl/factory/iterative.hh:76-109).
// One iteration is five kernels: (1) p update fused with the block-Jacobi apply,
// (2) SpMV fused with <rhat, v>, (3) s update fused with the block-Jacobi apply and ||s||^2,
// (4) SpMV fused with <t, s> and <t, t>, (5) x / r update with ||r||^2 and <rhat, r>.
// Every kernel starts by reading a device "done" flag and returns at once when the solve
// has converged or broken down, so a CUDA graph of several iterations can be replayed
// without a host round trip per iteration.  Reductions are deterministic.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "linalg.cuh"

namespace dcgpu {

// device scalar slots
enum KrylovSlot : int {
  KS_RHO = 0, KS_ALPHA = 1, KS_OMEGA = 2, KS_RHONEW = 3, KS_RV = 4, KS_TS = 5, KS_TT = 6,
  KS_RR = 7, KS_SS = 8, KS_BETA = 9, KS_TARGET = 10, KS_DONE = 11, KS_ITER = 12, KS_RR0 = 13,
  KS_FAULT = 14,    // single-launch solve: 1 when a grid-barrier wait gave up
  KS_BARRIER = 15,  // single-launch solve: the barrier's arrival counter and generation (2 x u32)
  KS_COUNT = 16
};
// KS_DONE values
constexpr double kDoneConverged = 1.0, kDoneBreakdown = 2.0, kDoneNonFinite = 3.0;

// ---------------------------------------------------------------- single-launch BiCGSTAB
// The whole preconditioned BiCGSTAB solve in ONE cooperative launch: the phases of an
// iteration are separated by grid-wide barriers instead of kernel boundaries, every block
// folds the per-block partial sums itself (same values, same order, so every block takes
// the same convergence decision), and the loop runs on the device until convergence,
// breakdown or max_it.  Same arithmetic per element as the five-kernel iteration below.
// On the SELL-32 operator with block size <= 2 an iteration has three phases: each SpMV
// forms the preconditioned vector it multiplies (D^-1 (r + beta (p - omega v)), then
// D^-1 (r - alpha v)) for every column it gathers, instead of reading it from a vector
// written in a phase of its own; the BSR operator keeps five phases.
// Each barrier wait is bounded in time; a wait that gives up sets sc[KS_FAULT] and the
// kernel returns.  Block Jacobi only (no multigrid cycle inside the kernel).
template <class T, class V>
struct FusedBicgArgs {
  int nrows = 0;
  const int32_t* rowptr = nullptr;  // BSR operator (used when sell is false)
  const int32_t* colidx = nullptr;
  Sell S{};                         // SELL-32 operator (used when sell is true)
  const V* vals = nullptr;          // operator values in the chosen layout
  const V* dinv = nullptr;          // block-Jacobi inverses
  T *x, *r, *rhat, *p, *v, *s, *t, *phat, *shat;
  T *p2, *v2;                       // second p and v buffers (the SELL variant alternates them)
  double* partial = nullptr;        // 5 * gridDim.x doubles
  double* sc = nullptr;             // device scalars (KrylovSlot)
  double rel = 0.0;
  int max_it = 0;
  // Mixed-precision iterative refinement around the solve (b64 null: a plain solve of r):
  // solve J z = b64 in fp64 to the relative residual rel, each correction by the solve above
  // in T on the scaled residual, to the relative reduction max(inner, rel / 2 / |r| * |b|).
  // vals64 holds J in the BSR layout of rowptr / colidx; r64 is fp64 scratch.
  const double* b64 = nullptr;
  double* z64 = nullptr;
  double* r64 = nullptr;
  const double* vals64 = nullptr;
  double inner = 1e-4;
  int max_refinements = 50;
};
// results of a refined solve: sc[KS_ITER] all inner iterations, sc[KS_REFINEMENTS] the
// corrections, sc[KS_RR] the final |r|^2 (fp64), sc[KS_DONE] 1 converged, 2 diverged (a
// non-finite residual, or a correction that broke down in its first iteration), 0 not
// converged within max_it iterations / max_refinements corrections
constexpr int KS_REFINEMENTS = KS_SS;
// Launch plan of the single-launch solve for block size bs: false when the device cannot
// run it (no cooperative launch, unsupported block size).  blocks is bounded by what is
// co-resident on the device and by the problem size; `slots` is the share of the device
// the grid holds, in units of which the device has `capacity` (co-resident blocks at the
// kernels' minimum occupancy), so that grids in flight together can be kept within it.
template <class T, class V>
bool fused_bicgstab_plan(int bs, bool sell, int nrows, int* blocks, int* slots, int* capacity);
// partial-sum doubles the solve needs for `blocks` blocks
inline int64_t fused_bicgstab_partials(int blocks) { return 5 * static_cast<int64_t>(blocks); }
// resets the barrier words and the fault flag, then launches the solve on `s`
template <class T, class V>
void fused_bicgstab(int bs, bool sell, int blocks, const FusedBicgArgs<T, V>& a, cudaStream_t s);
// Runs one grid-wide barrier that cannot complete (4 blocks, 50 ms limit): every block's wait
// must give up and flag it.  Returns non-zero on a CUDA error; gave_up_blocks receives the
// number of blocks that flagged, elapsed_ms the kernel's duration.
int barrier_selftest(double* gave_up_blocks, double* elapsed_ms);
// FP64 / FP32 fused multiply-add throughput of the current device in TFLOP/s (peaks.cu);
// returns non-zero on a CUDA failure
int fma_peaks(double* fp64_tflops, double* fp32_tflops);

template <class T>
struct KrylovVectors {
  T *x, *r, *rhat, *p, *v, *s, *t, *phat, *shat;
};

// r must hold the right-hand side; sets x = 0, rhat = r, p = v = 0 and the scalars;
// target = (rel * ||r||)^2
template <class T>
void krylov_init(const KrylovVectors<T>& k, int64_t n, double rel, ReduceScratch rs, double* sc, cudaStream_t s);

// one iteration (five launches); V is the matrix / preconditioner value type.  When `ev`
// is given, ev[0..1] bracket the first SpMV kernel and ev[2..3] the second.
// With `pc`, the preconditioner is pc->apply (a separate launch sequence) instead of the
// block-Jacobi inverse `dinv` fused into the update kernels.  With `sell`, the two SpMVs
// read `vals` in that SELL-32 layout instead of A's BSR layout.
class Preconditioner;

// Preconditioned CG (dune-istl CGSolver; also used for GeneralizedPCG / RestartedFCG /
// CompleteFCG, which coincide with CG for a fixed preconditioner).  cg_init: x = 0, z =
// M^-1 r, rho = <r, z>; one iteration: p = z + beta p; q = A p, alpha = rho / <p, q>;
// x += alpha p, r -= alpha q, z = M^-1 r, beta = <r, z>_new / rho.  Vectors: x, r, p,
// z in `s`, q in `v`.  Same device scalars, done flag and graph capture as BiCGSTAB.
template <class T, class V>
void cg_init(const Bsr& A, const V* dinv, const KrylovVectors<T>& k, double rel, ReduceScratch rs, double* sc,
             cudaStream_t s, const Preconditioner* pc = nullptr);
template <class T, class V>
void cg_iteration(const Bsr& A, const V* vals, const V* dinv, const KrylovVectors<T>& k, ReduceScratch rs,
                  double* sc, cudaStream_t s, const Preconditioner* pc = nullptr, const Sell* sell = nullptr);

template <class T, class V>
void krylov_iteration(const Bsr& A, const V* vals, const V* dinv, const KrylovVectors<T>& k, ReduceScratch rs,
                      double* sc, cudaStream_t s, cudaEvent_t* ev = nullptr, const Preconditioner* pc = nullptr,
                      const Sell* sell = nullptr);

}  // namespace dcgpu
