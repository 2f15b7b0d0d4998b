// Continuous batching of Krylov solves across concurrently running simulations.
//
// No counterpart in the reference (it runs one simulation per process, and its
// LinearSolver, dune/copasi/model/make_step_operator.hh:102-146, solves one system at a
// time).  Simulations served side by side each run their own Newton loop on their own
// host thread and CUDA stream; when one needs a block-Jacobi preconditioned BiCGSTAB solve
// it hands the system to a KrylovBatcher and waits.  The batcher's thread packs every
// system it holds -- different meshes, block sizes and lengths -- into one set of tile
// kernels: an instance is cut into tiles of 256 block rows, the tile table lists the tiles
// of all instances, and each of the five phase kernels of a BiCGSTAB iteration walks that
// table with a fixed grid.  Runs of 2, 4 and 8 iterations are captured once as CUDA graphs
// whose kernels read the table from device memory, so the same graphs serve every batch
// composition.  Between replays the batcher retires the instances that converged (their
// callers resume at once) and admits the systems that arrived meanwhile; new instances
// join the running batch instead of waiting for it to drain.
//
// Every instance's arithmetic is independent of the others: a tile's partial sums are
// formed by the same threads in the same order whatever block runs it, and an instance's
// partials are folded in tile order by whichever block finishes its last tile.  A result
// is therefore bitwise the same alone and in any mix.
#pragma once

#include <cstdint>
#include <memory>
#include <string>

#include <cuda_runtime.h>

#include "sell.cuh"

namespace dcgpu {

// One linear system A x = r handed to the batcher: block size bs (1..8), nrows block rows,
// A in the SELL-32 layout S with entry-interleaved values `vals`, block-Jacobi inverses
// `dinv` (nrows * bs * bs, row-major blocks), and the caller's Krylov vectors (nrows * bs
// each).  r holds the right-hand side on entry; the solution is left in x.
template <class T>
struct BatchSystem {
  int nrows = 0;
  int bs = 1;
  Sell S{};
  const T* vals = nullptr;
  const T* dinv = nullptr;
  T *x = nullptr, *r = nullptr, *rhat = nullptr, *p = nullptr, *v = nullptr, *s = nullptr, *t = nullptr,
    *phat = nullptr, *shat = nullptr;
};

struct BatchStats {
  int64_t solves = 0;        // systems solved
  int64_t replays = 0;       // graph replays (2, 4 or 8 iterations of every active instance)
  int64_t slot_replays = 0;  // sum over replays of the instances active in them
  int64_t iterations = 0;    // BiCGSTAB iterations of all solved systems
  int32_t max_active = 0;    // most instances in one replay
  double replay_s = 0.0;     // host time from the start of each replay's enqueue to its end
  double wait_s = 0.0;       // time the callers spent blocked in solve(), summed over calls
};

class KrylovBatcher {
 public:
  // max_slots: instances one batch holds at once (1..1024); systems beyond wait for a slot
  KrylovBatcher(int device, int max_slots);
  ~KrylovBatcher();
  KrylovBatcher(const KrylovBatcher&) = delete;
  KrylovBatcher& operator=(const KrylovBatcher&) = delete;

  // Solves sys to the relative residual reduction rel (in the 2-norm, dune-istl
  // BiCGSTABSolver semantics) within max_it iterations and blocks the calling thread until
  // it is done.  The batcher's stream first waits for the work enqueued on `caller` so far
  // (the operator, the inverses and the right-hand side); when the call returns, the solve
  // has completed on the device.  Returns 0 (converged), 1 (breakdown or a non-finite
  // value) or 3 (max_it reached), with the iterations in *iters; throws CudaError when a
  // CUDA call of the batch failed.
  int solve(const BatchSystem<float>& sys, cudaStream_t caller, double rel, int max_it, int* iters);
  int solve(const BatchSystem<double>& sys, cudaStream_t caller, double rel, int max_it, int* iters);

  BatchStats stats() const;
  // the replay grid the autotuner chose per batch size, per precision, as JSON
  std::string tuning() const;

  struct Impl;

 private:
  std::unique_ptr<Impl> impl_;
};

}  // namespace dcgpu
