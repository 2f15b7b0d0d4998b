// Aggregation algebraic multigrid on the block (BSR) Jacobian, applied as a V(1,1) cycle
// with damped block-Jacobi smoothing.
//
// The reference offers no multigrid (its preconditioners are dune-istl's Richardson,
// Jacobi, SSOR, SOR, Gauss-Seidel, ILU variants and BlockJacobi,
// dune/copasi/solver/istl/factory/preconditioner.hh:226-256); this is the GPU engine's
// preconditioner for stiff, diffusion-dominated stage systems (large D dt / h^2), where
// block Jacobi needs hundreds of Krylov iterations.
//
// Structure (once per model, on the host): the block-row graph is coarsened by greedy
// aggregation restricted to rows of the same compartment (a row and its not yet aggregated
// neighbours form an aggregate; leftovers join a neighbouring aggregate), level after level,
// until a level has at most `min_rows` rows.  Prolongation is piecewise constant per
// aggregate, so the Galerkin operator A_c = P^T A P is a sum of fine blocks; for every
// coarse block the list of fine blocks that add into it is precomputed.
// Values (every Newton iteration, on the device): coarse blocks are summed in a fixed
// order (deterministic), each level's block-Jacobi inverse is formed, and fp32 copies are
// kept for the mixed-precision Krylov path.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "linalg.cuh"
#include "model.hpp"

namespace dcgpu {

class Amg {
 public:
  Amg() = default;
  Amg(const Amg&) = delete;
  Amg& operator=(const Amg&) = delete;

  // rows of different `group` are never aggregated together
  void build(const std::vector<int32_t>& rowptr, const std::vector<int32_t>& colidx,
             const std::vector<int32_t>& diag, const std::vector<int32_t>& group, int bs, int max_levels = 10,
             int min_rows = 256);
  // Galerkin values and smoother inverses of every coarse level from the fine values
  // (fine_dinv: the fine block-Jacobi inverses already computed by the solver); with fp32,
  // float copies of every level as well (fine_vals32 / fine_dinv32 already converted)
  void setup(const double* fine_vals, const double* fine_dinv, const float* fine_vals32, const float* fine_dinv32,
             bool fp32, int* status, cudaStream_t s);
  // z = M^-1 r, one V(1,1)-cycle; no work when sc != nullptr and sc[done] != 0
  template <class T>
  void apply(const T* r, T* z, const double* sc, int done_slot, cudaStream_t s) const;

  int levels() const { return static_cast<int>(levels_.size()); }
  int64_t rows(int l) const { return levels_[l].nrows; }
  bool built() const { return !levels_.empty(); }

  double omega = 0.8;      // block-Jacobi damping
  int coarse_sweeps = 6;   // block-Jacobi sweeps on the coarsest level

 private:
  struct Level {
    int64_t nrows = 0, nnzb = 0;
    // pattern of this level (level 0: borrowed from the model)
    DeviceBuffer<int32_t> rowptr_o, colidx_o, diag_o;
    const int32_t* rowptr = nullptr;
    const int32_t* colidx = nullptr;
    const int32_t* diag = nullptr;
    // values of this level (level 0: borrowed from the solver)
    DeviceBuffer<double> val_o, dinv_o;
    DeviceBuffer<float> val32_o, dinv32_o;
    const double* val = nullptr;
    const double* dinv = nullptr;
    const float* val32 = nullptr;
    const float* dinv32 = nullptr;
    // aggregation to the next level
    DeviceBuffer<int32_t> agg, agg_ptr, agg_rows, gal_ptr, gal_src;
    // work vectors (x: correction, t: residual), fp64 and fp32
    DeviceBuffer<double> x, t, rc;
    DeviceBuffer<float> x32, t32, rc32;
  };
  std::vector<Level> levels_;
  int bs_ = 1;
};

}  // namespace dcgpu
