// Device-side data structures shared by the assembly kernels and the host driver.
#pragma once

#include <cstdint>

#include "bytecode.hpp"
#include "lookup.hpp"

namespace dcgpu {

// One compiled expression program resident in device memory.
struct DevProgram {
  const Instr* code = nullptr;
  const double* consts = nullptr;
  const float* consts32 = nullptr;  // the same constants rounded to FP32 (FP32 interpreter)
  const uint16_t* inputs = nullptr;
  const uint8_t* outputs = nullptr;
  int ncode = 0, ninputs = 0, noutputs = 0, nregs = 0;
};

// Lookup tables of the parser context: 1-D interpolation tables, tabulated functions and
// grayscale images
struct DevTables {
  const double* x = nullptr;
  const double* y = nullptr;
  const int* off = nullptr;
  const int* len = nullptr;
  const FnTableDesc* ft = nullptr;   // tabulated functions, values in ftg
  const double* ftg = nullptr;
  const ImageDesc* im = nullptr;     // images, pixels in imp
  const double* imp = nullptr;
};

// Volume term kinds (residual and Jacobian of local_operator.hh:417-707).
enum TermKind : uint8_t {
  // residual
  R_REACTION = 0,     // scalar -= out
  R_STORAGE,          // scalar += u_test * out
  R_VELOCITY,         // flux += out[0..dim) * u_test
  R_DIFF_SCALAR,      // flux -= out * grad u_trial
  R_DIFF_TENSOR,      // flux -= T(out[0..dim^2)) grad u_trial
  // Jacobian
  J_MASS,             // J[a,test][b,trial] += out * phi_a phi_b
  J_MASS_U,           // J[a,test][b,trial] += out * u_test * phi_a phi_b
  J_STORAGE_SELF,     // J[a,test][b,test]  += out * phi_a phi_b
  J_VELOCITY,         // J[a,test][b,test]  -= phi_a (v . G_b)
  J_VELOCITY_JAC,     // J[a,test][b,trial] -= phi_a ((out * u_test) . G_b)
  J_DIFF_SCALAR,      // J[a,test][b,trial] += out (G_a . G_b)
  J_DIFF_TENSOR,      // J[a,test][b,trial] += (T G_a) . G_b
  J_DIFFJAC_SCALAR,   // J[a,test][b,trial] += phi_a (out grad u_trial) . G_b
  J_DIFFJAC_TENSOR,   // J[a,test][b,trial] += phi_a (T grad u_trial) . G_b
  // faces
  F_OUTFLOW,          // r[k,test] += out * psi_k
  F_OUTFLOW_JAC,      // J[k,test][l,trial@side] += out * psi_k psi_l
};

struct Term {
  uint8_t kind;
  uint8_t form;     // 0 = mass form (scaled by cm), 1 = stiffness form (scaled by ca)
  uint8_t test;     // local species index (compartment of the element / face side)
  uint8_t trial;    // local species index of the trial / gradient species
  uint8_t side;     // faces: 0 = trial lives on this side, 1 = on the other side
  uint8_t slot;     // volume Jacobian terms: index of the (test, trial) pair in the element output
  uint16_t out;     // first program output
  uint16_t coef;    // Jacobian terms: offset into the per-thread coefficient array
  uint16_t pad2;
};

constexpr int kMaxDevRegisters = 64;   // register file of the device interpreter
constexpr int kMaxCoefficients = 192;  // per-element Jacobian coefficient storage

// Launch parameters for the volume assembly of one compartment.
struct VolumeParams {
  const double* coords;      // nv * dim
  const int32_t* verts;      // ne * nl (coloured order)
  const int32_t* nodes;      // ne * nl block-row index of each local vertex
  const int32_t* bpos;       // ne * nl * nl block index in the BSR pattern
  const Term* res_terms;
  const Term* jac_terms;
  int n_res_terms, n_jac_terms;
  DevProgram prog;           // outputs for residual (and Jacobian when assembling it)
  DevTables tables;
  const double* x;           // state, node-major with block size bs
  double* r;                 // residual accumulator (may be null)
  double* J;                 // BSR values accumulator (may be null)
  int bs;                    // block size
  int species_offset;        // model-global index of local species 0
  double t, cm, ca;          // time, mass-form scale, stiffness-form scale
  double fd_eps;             // numerical Jacobian: relative perturbation
  // element outputs of k_volume (gathered into r / J afterwards)
  double* er;                // residual: (k * nl + a) * ns + s
  double* ej;                // Jacobian: ((k * nl + a) * nl + b) * n_slots + slot
  int n_slots;               // distinct (test, trial) pairs of the Jacobian terms
  int all_mass;              // every Jacobian term is mass-type: symmetric element matrix
  // matrix-free Jacobian products (mode kVolumeJacobianApply): the direction v (node-major,
  // block size bs) and the block position test * bs + trial of every Jacobian slot; the
  // element's J v goes to er like a residual
  const double* v;
  const int32_t* slot_pos;
  int jac_f32;               // element Jacobian in fp32 (ej then holds floats)
  // work the kernel may skip (uniform flags set from the program inputs and term kinds)
  int need_pos;              // a program reads position_*
  int need_grad;             // a program reads a gradient or a term takes one
  int has_flux;              // a residual term contributes a flux (velocity / diffusion)
  int need_vol;              // a program reads entity_volume
  int ncoef;                 // Jacobian coefficients per element of the jac_terms (0 without)
};

// A thread's slice of a block-wide shared-memory array: element i at p[i * stride] (stride =
// block size, so the threads of a warp touch consecutive words).  The volume kernel keeps
// the interpreter's register file and the element's Jacobian coefficients there: indexed
// at run time, as local arrays they lived in local memory and spilled to L2 and DRAM.
template <class F>
struct Strided {
  F* p;
  int stride;
  __device__ __forceinline__ F& operator[](int i) const { return p[i * stride]; }
};
// the same array read through a conversion to U (fp64 coefficients of an fp32 element matrix)
template <class F, class U>
struct StridedCast {
  const F* p;
  int stride;
  __device__ __forceinline__ U operator[](int i) const { return static_cast<U>(p[i * stride]); }
};

struct FaceParams {
  const double* coords;
  const int32_t* fverts;     // nf * dim face vertices
  const int32_t* node_in;    // nf * dim block rows of the face vertices, side 0 compartment
  const int32_t* node_out;   // nf * dim block rows, side 1 compartment (or -1)
  const int32_t* bpos;       // nf * 4 * dim * dim : (in,in) (in,out) (out,in) (out,out)
  const double* normal;      // nf * dim unit normal pointing from side 0 to side 1
  const double* ielem;       // nf integration element (edge length / twice the triangle area)
  const double* fvolume;     // nf face measure (entity_volume)
  const int32_t* elem_in;    // nf elements (for gradients)
  const int32_t* elem_out;
  const int32_t* cells;      // mesh cells (nl per element)
  const int32_t* vnode[2];   // vertex -> block row of each side's compartment (-1 if absent)
  const Term* terms[2];      // per side
  int n_terms[2];
  DevProgram prog[2];        // per side
  DevTables tables;
  const double* x;
  double* r;
  double* J;
  // matrix-free Jacobian products (mode kFaceJacobianApply): y += J_face v
  const double* v;
  double* y;
  int bs;
  int species_offset[2];     // model-global species index of local species 0, per side
  int ns[2];
  double t, ca;
};

}  // namespace dcgpu
