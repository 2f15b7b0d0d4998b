// Aggregation algebraic multigrid on the block (BSR) Jacobian, applied as one V(1,1) cycle
// per preconditioner application.
//
// The reference offers no multigrid (its preconditioners are dune-istl's Richardson,
// Jacobi, SSOR, SOR, Gauss-Seidel, ILU variants and BlockJacobi,
// dune/copasi/solver/istl/factory/preconditioner.hh:88-112); this is the GPU engine's
// preconditioner for stiff, diffusion-dominated stage systems (large D dt / h^2), where
// block Jacobi needs hundreds of Krylov iterations.
//
// Structure (once per pattern, on the device): each level's block-row graph, restricted to
// edges between rows of the same compartment, is coarsened around a distance-k maximal
// independent set (graph.hpp): roots and the rows that join them form the aggregates.
// Coarsening stops at a level small enough for the dense direct solve (at most
// kDenseMax unknowns), at `max_levels`, or when it stalls.  Prolongation is piecewise
// constant per aggregate, so the Galerkin operator A_c = P^T A P is a sum of fine blocks:
// for every coarse block the list of the fine blocks that add into it is precomputed.
// Values (every Newton iteration, on the device): coarse blocks are summed in a fixed order
// (deterministic), every level's smoother is set up, and the coarsest operator is factored
// by a dense FP64 LU with partial pivoting and inverted.  The cycle reads SELL-32 copies of
// the level operators (sell.cuh) in the precision of the Krylov solve (fp32 in the
// mixed-precision path).
// Smoothers: damped block Jacobi, block L1-Jacobi (the diagonal block plus the absolute row
// sums of the off-diagonal blocks on its diagonal), multicolour block Gauss-Seidel (forward
// sweep before the coarse correction, backward sweep after it: a symmetric cycle), or
// multicolour block ILU(0) (x = M^-1 r before, x += M^-1 (r - A x) after).
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "graph.hpp"
#include "linalg.cuh"
#include "mcolor.hpp"
#include "model.hpp"
#include "precond.hpp"

namespace dcgpu {

class Amg : public Preconditioner {
 public:
  enum class Smoother { Jacobi, L1Jacobi, GaussSeidel, Ilu0 };
  // largest coarsest level (unknowns) solved by the dense LU
  static constexpr int kDenseMax = 128;
  // levels with fewer rows use the warp-per-row kernels (default of warp_rows_below)
  static constexpr int64_t kWarpRowsBelow = 65536;

  Amg() = default;
  Amg(const Amg&) = delete;
  Amg& operator=(const Amg&) = delete;

  // hierarchy of the pattern (device arrays, borrowed for level 0); rows of different
  // `group` (device, null: one group) are never aggregated together
  void build(int64_t nrows, int bs, int64_t nnzb, const int32_t* rowptr, const int32_t* colidx, const int32_t* diag,
             const int32_t* group, cudaStream_t s);
  // Galerkin values, smoothers and the coarse factorisation from the fine values
  // (fine_dinv: the fine block-Jacobi inverses already computed by the solver).  The cycle
  // then runs in fp32 (fp32 true; fine_dinv32: the inverses already rounded) or in fp64.
  // With fine_sell / fine_sell32 (fp32 only), the finest level's products read that SELL-32
  // copy of the fine operator (the Krylov solve's own) instead of a copy of their own.
  void setup(const double* fine_vals, const double* fine_dinv, const float* fine_dinv32, bool fp32, int* status,
             cudaStream_t s, const Sell* fine_sell = nullptr, const float* fine_sell32 = nullptr);
  // z = M^-1 r, one V(1,1)-cycle; no work when sc != nullptr and sc[done] != 0
  void apply(const double* r, double* z, const double* sc, int done_slot, cudaStream_t s) const override;
  void apply(const float* r, float* z, const double* sc, int done_slot, cudaStream_t s) const override;

  int levels() const { return static_cast<int>(levels_.size()); }
  // the hierarchy as a JSON object: smoother, rows / blocks / kernel kind per level
  std::string describe() const;
  int64_t rows(int l) const { return levels_[l].nrows; }
  int64_t blocks(int l) const { return levels_[l].nnzb; }
  bool built() const { return !levels_.empty(); }
  bool dense_coarse() const { return dense_n_ > 0; }
  int colors(int l) const { return levels_[l].gs ? levels_[l].gs->colors() : 0; }
  // aggregate of every row of level l (l + 1 < levels()), the values of level l (fp64), the
  // inverse of the coarsest operator (row-major, dense_coarse() only): for tests
  std::vector<int32_t> aggregates_host(int l) const { return levels_[l].agg.download(); }
  std::vector<double> values_host(int l) const;
  std::vector<int32_t> rowptr_host(int l) const;
  std::vector<int32_t> colidx_host(int l) const;
  std::vector<double> coarse_inverse_host() const { return dinvd_.download(); }

  // parameters (read before build)
  Smoother smoother = Smoother::Jacobi;
  double omega = 0.85;       // smoother relaxation
  int coarse_sweeps = 6;     // smoother sweeps on a coarsest level too large for the dense solve
  int max_levels = 10;
  int64_t coarsen_target = 0;  // stop coarsening at this many rows (0: the dense solve's limit)
  int mis_distance = 2;      // aggregation around a distance-1 or distance-2 independent set
  double correction = 1.0;   // scale of the coarse-grid correction x += correction * P xc
  // (L1-)Jacobi smoothing: post-smoothing on the finest level too (false: V(1,0) there, one
  // pass over the finest operator less per cycle)
  bool finest_post_smoothing = true;
  // (L1-)Jacobi smoothing: the top w_levels levels take two coarse-grid corrections per visit
  // (a W-cycle there; 0: V-cycle)
  int w_levels = 0;
  int64_t warp_rows_below = kWarpRowsBelow;

 private:
  struct Level {
    int64_t nrows = 0, nnzb = 0;
    // pattern of this level (level 0: borrowed from the model)
    const int32_t* rowptr = nullptr;
    const int32_t* colidx = nullptr;
    const int32_t* diag = nullptr;
    const int32_t* group = nullptr;
    CoarseStructure own;  // this level's pattern when it is a coarse level
    // BSR values of this level and their block-Jacobi inverses (level 0: borrowed from the
    // solver); the cycle's products read the SELL-32 copy in the precision of the last setup
    DeviceBuffer<double> val_o, dinv_o;
    DeviceBuffer<float> dinv32_o;
    const double* val = nullptr;
    const double* dinv = nullptr;
    const float* dinv32 = nullptr;
    // products: lane per row on a SELL-32 copy (large levels), or warp per row on the BSR
    // values (levels below warp_rows_below rows, where a lane per row leaves the GPU idle
    // and each lane would walk a long coarse row alone)
    bool warp_rows = false;
    SellStructure sell;
    bool ext = false;  // level 0 reading the caller's SELL-32 copy (ext_view, ext_sv32)
    Sell ext_view{};
    const float* ext_sv32 = nullptr;
    DeviceBuffer<double> sv64;
    DeviceBuffer<float> sv32, val32_o;
    // smoother inverses (L1-Jacobi: own; else the block-Jacobi inverses above)
    DeviceBuffer<double> sinv_o;
    DeviceBuffer<float> sinv32_o;
    std::unique_ptr<ColorPrecond> gs;  // Gauss-Seidel / ILU(0) smoother of this level (multicolour)
    // aggregation to the next level (agg_ptr / agg_rows / gal_* live in the next level's own)
    DeviceBuffer<int32_t> agg;
    // work vectors: x the correction, t the smoothed iterate / residual, rc the right-hand side
    DeviceBuffer<double> x, t, rc, w;  // w: the ILU(0) smoother's correction
    DeviceBuffer<float> x32, t32, rc32, w32;
  };
  template <class T>
  void cycle(int l, const T* r, T* x, const double* sc, int slot, cudaStream_t s) const;
  template <class T>
  void apply_t(const T* r, T* z, const double* sc, int done_slot, cudaStream_t s) const;

  std::vector<Level> levels_;
  int bs_ = 1;
  bool fp32_ = false;  // precision of the last setup
  // dense coarsest solve: n unknowns, the operator's inverse (row-major) in fp64 / fp32
  int dense_n_ = 0;
  DeviceBuffer<double> dense_, dinvd_;
  DeviceBuffer<float> dinvf_;
  DeviceBuffer<int32_t> dense_piv_;
};

}  // namespace dcgpu
