// Multicolour block preconditioners: SSOR, SOR / Gauss-Seidel, ILU(0) and DILU on the
// block (BSR) Jacobian, in the order of a colouring of the block-row graph.
//
// The reference's registry (dune/copasi/solver/istl/factory/preconditioner.hh:94-112) builds
// dune-istl's SeqSSOR (its default), SeqSOR, SeqGS, SeqILU, SeqDILU and SeqILDL.  Those sweep
// the rows in their natural order, one row after another.  Here the rows are ordered by
// colour instead (rows of one colour are never adjacent), so every colour is one parallel
// launch: a sweep is a loop over the colours, and the ILU(0) / DILU factorisations are
// computed colour by colour in the same way.  The preconditioner is the same kind of
// operator in another row order; the converged Krylov solution is the same to its tolerance.
//
// Parameters follow dune-istl: `iterations` (SSOR / SOR sweeps, default 1) and `relaxation`
// (omega, default 1; ILU and DILU scale their result by it).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "graph.hpp"
#include "model.hpp"
#include "precond.hpp"

namespace dcgpu {

class ColorPrecond : public Preconditioner {
 public:
  enum class Kind { Ssor, Sor, Ilu0, Dilu };

  ColorPrecond() = default;
  ColorPrecond(const ColorPrecond&) = delete;
  ColorPrecond& operator=(const ColorPrecond&) = delete;

  // colouring of the pattern's block-row graph (once per pattern); the pattern arrays are
  // borrowed and must outlive this object
  void build(Kind kind, int64_t nrows, int bs, int64_t nnzb, const int32_t* rowptr, const int32_t* colidx,
             const int32_t* diag, cudaStream_t s);
  // numeric set-up for new values: vals / dinv are the operator and its block-Jacobi
  // inverses (fp64; dinv32 the inverses rounded to fp32, needed with fp32; borrowed until the
  // next setup).  The sweeps then run in fp32 (fp32 true) or fp64 and read SELL-32 copies
  // (sell.cuh) of the operator or factors made here.  ILU(0) and DILU factor here (in fp64);
  // status[0] != 0 on a singular pivot block.
  // With sell_ext / sv32_ext (fp32, SSOR / SOR / DILU), the sweeps read that SELL-32 copy
  // of the operator (the Krylov solve's own) instead of a copy of their own.
  void setup(const double* vals, const double* dinv, const float* dinv32, bool fp32, int* status, cudaStream_t s,
             const Sell* sell_ext = nullptr, const float* sv32_ext = nullptr);
  void apply(const double* r, double* z, const double* sc, int done_slot, cudaStream_t s) const override;
  void apply(const float* r, float* z, const double* sc, int done_slot, cudaStream_t s) const override;

  // One SOR sweep of A z = r with the values of the last setup and relaxation omega:
  // colours ascending (forward) or descending; from_zero (forward only) takes z = 0 on entry
  // and reads only the earlier colours.  The multigrid smoother.
  template <class T>
  void sor_sweep(const T* r, T* z, bool forward, bool from_zero, const double* sc, int done_slot,
                 cudaStream_t s) const;

  Kind kind() const { return kind_; }
  // JSON object: kind, colours, relaxation, iterations
  std::string describe() const;
  int colors() const { return static_cast<int>(offsets_.size()) - 1; }
  bool built() const { return !offsets_.empty(); }
  // colour of every block row and the rows in colour order (tests)
  std::vector<int32_t> colour_host() const { return colour_.download(); }
  std::vector<int32_t> perm_host() const { return perm_.download(); }

  double omega = 1.0;
  int iterations = 1;

 private:
  template <class T>
  void apply_t(const T* r, T* z, const double* sc, int done_slot, cudaStream_t s) const;
  template <class T>
  void sweep_color(int mode, int c, const T* vals, const T* dmat, const T* r, T* z, const double* sc, int done_slot,
                   cudaStream_t s) const;

  Kind kind_ = Kind::Ssor;
  int64_t n_ = 0, nnzb_ = 0;
  int bs_ = 1;
  const int32_t* rowptr_ = nullptr;
  const int32_t* colidx_ = nullptr;
  const int32_t* diag_ = nullptr;
  DeviceBuffer<int32_t> colour_, perm_, ipos_;
  std::vector<int64_t> offsets_;  // colour c: perm[offsets_[c] .. offsets_[c + 1])
  SellStructure sell_;
  bool fp32_ = false;  // precision of the last setup
  Sell ext_view_{};
  const float* ext_sv32_ = nullptr;  // borrowed operator copy (null: own)
  // borrowed block-Jacobi inverses
  const double* dinv_ = nullptr;
  const float* dinv32_ = nullptr;
  // owned: the operator (SSOR / SOR / DILU) or the ILU(0) factors (L / U blocks in the
  // pattern) in the SELL-32 layout; ILU(0) / DILU inverse pivot blocks per row
  DeviceBuffer<double> lu_, dfac_, sv64_;
  DeviceBuffer<float> dfac32_, sv32_;
};

// Richardson: z = omega r (dune-istl Richardson, the registry's matrix-free entry)
class RichardsonPrecond : public Preconditioner {
 public:
  double omega = 1.0;
  int64_t n = 0;
  void apply(const double* r, double* z, const double* sc, int done_slot, cudaStream_t s) const override;
  void apply(const float* r, float* z, const double* sc, int done_slot, cudaStream_t s) const override;
};

}  // namespace dcgpu
