// Preconditioners applied by a separate sequence of launches between the Krylov phases
// (the block-Jacobi inverse is fused into the Krylov kernels themselves and needs none).
//
// The reference builds its preconditioner from a registry keyed by
// linear_solver.preconditioner.type (dune/copasi/solver/istl/factory/preconditioner.hh:88-118):
// Richardson, Jacobi, SSOR (the default), SOR, GaussSeidel, DILU, ILU, ILDL, BlockJacobi
// and InverseOperator.  The engine's implementations derive from this interface; the
// Krylov solvers call apply() once per preconditioner application.
#pragma once

#include <cuda_runtime.h>

namespace dcgpu {

class Preconditioner {
 public:
  virtual ~Preconditioner() = default;
  // z = M^-1 r on the stream s.  When sc is not null every launch starts by reading
  // sc[done_slot] and does no work once it is non-zero (a converged solve replayed from a
  // CUDA graph).  r and z do not alias.
  virtual void apply(const double* r, double* z, const double* sc, int done_slot, cudaStream_t s) const = 0;
  virtual void apply(const float* r, float* z, const double* sc, int done_slot, cudaStream_t s) const = 0;
};

}  // namespace dcgpu
