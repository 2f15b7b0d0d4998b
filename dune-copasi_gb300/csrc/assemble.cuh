// P1 residual / Jacobian assembly kernels (sm_103a).
//
// One thread per element of one colour class: the element gathers its vertex
// coordinates and coefficients, evaluates the compiled expression program at each
// quadrature point, accumulates its local residual and Jacobian coefficients, and adds
// them into the global residual / BSR values.  Elements of one colour share no vertex,
// so the read-modify-write scatter is race-free without atomics; the colour classes run
// as consecutive launches.  Restates local_operator.hh:417-491 (residual) and :541-707
// (analytic Jacobian); the face kernel restates :777-971 and :973-1203.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "device.cuh"

namespace dcgpu {

// mode bit 1: residual, bit 2: Jacobian; kVolumeNumericalJacobian: Jacobian by forward
// differences of the residual terms (params.prog / res_terms must be the residual program)
constexpr int kVolumeNumericalJacobian = 4;
// matrix-free Jacobian products: mode kVolumeJacobianApply | 2 evaluates each element's
// Jacobian and writes J_e v_e into the residual records (params.v, params.slot_pos);
// launch_faces with kFaceJacobianApply adds the face Jacobians times params.v to params.y
constexpr int kVolumeJacobianApply = 8;
constexpr int kFaceJacobianApply = 8;
void launch_volume(int dim, int ns, const VolumeParams& p, int begin, int end, int mode,
                   cudaStream_t stream);
void launch_faces(int dim, const FaceParams& p, int begin, int end, int mode, cudaStream_t stream);
// y = v on the unit rows of the Jacobian: the padded species slots of every block row
// (row_ns may be null: no padding) and the constrained DOFs
void launch_unit_rows_apply(const int8_t* row_ns, int64_t nrows, int bs, const int64_t* cons, int64_t ncons,
                            const double* v, double* y, cudaStream_t stream);
// numerical Jacobian of the outflow terms (forward differences of the face residuals) added to p.J
void launch_faces_fd(int dim, const FaceParams& p, int begin, int end, double eps, cudaStream_t stream);
// volume assembly is two-phase: k_volume writes per-element outputs (er / ej of
// VolumeParams), these gathers add them into r / J per node / block in list order
void launch_gather_residual(double* r, int bs, int ns, int64_t node_begin, int64_t nnodes, const int64_t* ptr,
                            const int32_t* list, const double* er, cudaStream_t stream);
// (f32: the element values are floats, summed in fp32).  Optional fused outputs of a gather
// that covers every entry of J: `overwrite` takes `base` (the static operator, or zero when
// null) in place of J's old value, and `sell` receives each final value rounded to fp32 at
// SELL-32 slot sell_bpos[block] (the mixed-precision operator copy, without a conversion pass).
struct JacobianGatherOut {
  int overwrite = 0;
  const double* base = nullptr;
  float* sell = nullptr;
  const int64_t* sell_bpos = nullptr;
};
void launch_gather_jacobian(double* J, int bs, int nslot, const int32_t* slot_pos, int64_t block_begin,
                            int64_t nblocks, const int64_t* ptr, const int32_t* list, const double* ej, bool f32,
                            cudaStream_t stream, const JacobianGatherOut& out = JacobianGatherOut{});
// The covering gather for a compartment whose dynamic slots are only some of the bs x bs
// entries of each block: every entry of every block of [block_begin, block_begin + nblocks)
// becomes base (out.overwrite's base, or zero) plus its dynamic slot's element values (slot m
// sits at entry slot_pos_host[m]); out.sell, when set, receives the fp32 copy.
void launch_gather_jacobian_full(double* J, int bs, int nslot, const std::vector<int32_t>& slot_pos_host,
                                 int64_t block_begin, int64_t nblocks, const int64_t* ptr, const int32_t* list,
                                 const double* ej, bool f32, cudaStream_t stream, const JacobianGatherOut& out);
// J[diag[i]] block gets identity in the padded slots s >= ns_of_row (rows of compartments
// with fewer species than the block size)
void launch_pad_identity(const int32_t* diag, const int8_t* row_ns, int nrows, int bs, double* J,
                         double value, cudaStream_t stream);
// constrained entries idx[0..n) (blocked vector index): op 0 sets v[idx] = val, op 1 zeroes them
void launch_constraints(double* v, const int64_t* idx, const double* val, int64_t n, int op, cudaStream_t stream);
struct ConstraintRows {
  const int32_t* rowptr;
  const int32_t* diag;
};
// the constrained rows of the BSR Jacobian become unit rows
void launch_constraint_rows(double* J, const ConstraintRows& cr, const int64_t* idx, int64_t n, int bs,
                            cudaStream_t stream);

}  // namespace dcgpu
