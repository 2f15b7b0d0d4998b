// Model setup: configuration -> mesh, compartments, species, DOF blocks, BSR pattern,
// colour classes, compiled expression programs and term tables, all resident on the
// device.
//
// Mirrors DiffusionReaction::make_model / ModelMultiCompartment (dune/copasi/model/
// diffusion_reaction/factory.hh:46-136, model_multi_compartment.impl.hh:55-92) and the
// functor tree of local_equations.hh:617-700 built through
// functor_factory_parser.impl.hh:25-182.  DOF layout (model_multi_compartment_traits.hh:
// 16-23): compartment-major, vertices ascending inside a compartment, the species of the
// compartment interleaved per vertex.  On the device every (compartment, vertex) pair is
// one block row of size bs = max species per compartment (padded slots carry an identity
// diagonal and a zero residual).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "device.cuh"
#include "expr.hpp"
#include "ini.hpp"
#include "linalg.cuh"
#include "mesh.hpp"
#include "volume_jit.hpp"

namespace dcgpu {

class CudaError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};
void cuda_check(cudaError_t e, const char* what);

// Device bytes held by the DeviceBuffers the calling host thread allocated (the request
// server measures a simulation's footprint with it: each runs on its own thread)
int64_t& device_bytes_this_thread();

template <class T>
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t n) { resize(n); }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  DeviceBuffer(DeviceBuffer&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
  DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) { release(); p_ = o.p_; n_ = o.n_; o.p_ = nullptr; o.n_ = 0; }
    return *this;
  }
  ~DeviceBuffer() { release(); }
  void resize(size_t n) {
    release();
    if (n) {
      cuda_check(cudaMalloc(&p_, n * sizeof(T)), "cudaMalloc");
      device_bytes_this_thread() += static_cast<int64_t>(n * sizeof(T));
    }
    n_ = n;
  }
  void upload(const std::vector<T>& h) {
    resize(h.size());
    if (n_) cuda_check(cudaMemcpy(p_, h.data(), n_ * sizeof(T), cudaMemcpyHostToDevice), "upload");
  }
  std::vector<T> download() const {
    std::vector<T> h(n_);
    if (n_) cuda_check(cudaMemcpy(h.data(), p_, n_ * sizeof(T), cudaMemcpyDeviceToHost), "download");
    return h;
  }
  T* get() const { return p_; }
  size_t size() const { return n_; }

 private:
  void release() {
    if (p_) {
      cudaFree(p_);
      device_bytes_this_thread() -= static_cast<int64_t>(n_ * sizeof(T));
    }
    p_ = nullptr;
    n_ = 0;
  }
  T* p_ = nullptr;
  size_t n_ = 0;
};

struct ReduceResult {
  std::string key;
  double value = 0.0;
  bool error = false;
  bool warn = false;
};

struct SpeciesInfo {
  std::string name;
  int comp = 0;   // compartment index
  int local = 0;  // index inside the compartment
  int global = 0; // model-wide index
};

// one compiled program + its device copy
struct ProgramBundle {
  Program host;
  DeviceBuffer<Instr> code;
  DeviceBuffer<double> consts;
  DeviceBuffer<float> consts32;
  DeviceBuffer<uint16_t> inputs;
  DeviceBuffer<uint8_t> outputs;
  DevProgram view() const;
  void upload();
};

struct VolumeGroup {
  int comp = 0, ns = 0;
  int64_t ne = 0;
  std::vector<int> color_offsets;  // colour c: [off[c], off[c+1])
  DeviceBuffer<int32_t> verts, nodes, bpos;
  ProgramBundle prog_static, prog_res, prog_all;
  std::vector<Term> static_terms;                          // for prog_static (Jacobian terms)
  std::vector<Term> res_terms_r, res_terms_a, jac_terms;   // for prog_res / prog_all
  DeviceBuffer<Term> d_static, d_res_r, d_res_a, d_jac;
  bool has_mass = false, has_stiffness = false;            // dynamic terms present
  bool static_mass = false, static_stiffness = false;      // static terms present
  // two-phase assembly: Jacobian slots (distinct test/trial pairs) of the static and the
  // dynamic term lists, and the gather lists of the compartment's nodes and blocks
  int slots_static = 0, slots_dyn = 0;
  bool static_all_mass = false, dyn_all_mass = false;
  DeviceBuffer<int32_t> slot_pos_static, slot_pos_dyn;     // test * bs + trial per slot
  std::vector<int32_t> slot_pos_dyn_host;
  int64_t node_begin = 0, nnodes = 0, block_begin = 0, nblocks = 0;
  DeviceBuffer<int64_t> rlist_ptr, blist_ptr;
  DeviceBuffer<int32_t> rlist, blist;                     // k * nl + a ; (k * nl + a) * nl + b
  std::shared_ptr<const JitVolume> jit;                   // run-time compiled kernels, or null
};

struct FaceGroup {
  int comp[2] = {-1, -1};
  bool boundary = false;
  int64_t nf = 0;
  std::vector<int> color_offsets;
  DeviceBuffer<int32_t> fverts, node_in, node_out, bpos, elem_in, elem_out;
  DeviceBuffer<double> normal, ielem, fvolume;
  ProgramBundle prog[2];
  std::vector<Term> terms[2];
  DeviceBuffer<Term> d_terms[2];
};

// uniform skip flags of the volume kernel for one program and its term lists, and the
// number of per-element Jacobian coefficients of the terms
void set_volume_flags(VolumeParams& p, const Program& prog, const std::vector<Term>& res, const std::vector<Term>& jac,
                      int dim);

class Model {
 public:
  Model(const std::string& ini_text, const std::string& overrides);
  ~Model() = default;

  // configuration
  Ini cfg;
  ParserContext ctx;
  Mesh mesh;
  int dim = 2;
  std::vector<std::string> comp_names;
  std::vector<int32_t> elem_comp;              // compartment of each element (-1: none)
  std::vector<SpeciesInfo> species;
  std::vector<int> ns;                          // species per compartment
  std::vector<int> species_offset;              // global index of the first species of each compartment
  bool is_linear = false;
  bool numerical_jacobian = false;
  // volume kernels: "compiled" (run-time compiled for the model's programs), "off", or
  // "interpreter (<reason>)" when the compilation was asked for and could not be had
  std::string jit_status = "off";
  // state-dependent (dynamic) terms: any in the mass form; any reading the time
  bool dynamic_mass = false, dynamic_time = false;
  double fd_eps = 1e-7;
  int bs = 1;

  // block rows
  int64_t nnodes = 0;
  int64_t ndof = 0;                             // reference DOF count (no padding)
  std::vector<int64_t> comp_node_offset;
  std::vector<std::vector<int32_t>> comp_vertices;  // ascending global vertex ids per compartment
  std::vector<std::vector<int32_t>> comp_vnode;     // vertex -> block row (-1 if absent)
  std::vector<int8_t> row_ns;                   // species count of each block row

  // BSR pattern
  std::vector<int32_t> rowptr, colidx, diag;
  DeviceBuffer<int32_t> d_rowptr, d_colidx, d_diag;
  DeviceBuffer<int8_t> d_row_ns;
  DeviceBuffer<int64_t> d_ref2blk;  // reference DOF index -> blocked state index
  bool padded = false;

  // geometry on the device
  DeviceBuffer<double> d_coords;
  DeviceBuffer<int32_t> d_cells;
  std::vector<DeviceBuffer<int32_t>> d_comp_vnode;
  DeviceBuffer<double> d_tab_x, d_tab_y;
  DeviceBuffer<int> d_tab_off, d_tab_len;
  DeviceBuffer<FnTableDesc> d_ftab_desc;
  DeviceBuffer<double> d_ftab_val;
  DeviceBuffer<ImageDesc> d_img_desc;
  DeviceBuffer<double> d_img_px;
  DevTables tables{};

  std::vector<VolumeGroup> vgroups;
  std::vector<FaceGroup> fgroups;
  // element outputs of the volume kernel (sized for the largest group; groups run in order)
  DeviceBuffer<double> d_er, d_ej;

  // static parts of the operator, assembled once: mass-form and stiffness-form BSR values
  DeviceBuffer<double> d_Ms, d_Ks;
  bool has_Ms = false, has_Ks = false;
  // cm Ms + ca Ks for the last (cm, ca) a Jacobian was assembled with: a DIRK stage keeps
  // its (cm, ca) for all its Newton iterations, so one combination serves the stage's
  // Jacobian copies and residual products
  mutable DeviceBuffer<double> d_Cs;
  mutable double cs_cm = 0.0, cs_ca = 0.0;
  mutable bool cs_valid = false;

  // Dirichlet constraints: blocked vector indices (ascending) and values
  std::vector<int64_t> cons_idx;
  std::vector<double> cons_val;
  int64_t n_constraints = 0;
  DeviceBuffer<int64_t> d_cons_idx;
  DeviceBuffer<double> d_cons_val;
  void apply_constraints(double* x, cudaStream_t s) const;   // x[idx] = val
  void constrain_residual(double* r, cudaStream_t s) const;  // r[idx] = 0
  void constrain_jacobian(double* J, cudaStream_t s) const;  // unit rows

  // transform/reduce operators of a reduce section on the blocked state x (device)
  std::vector<ReduceResult> reduce(const double* x, double t, const Ini& reduce_cfg, cudaStream_t s) const;
  mutable DeviceBuffer<int32_t> d_red_cells, d_red_nodes, d_red_comp;
  mutable DeviceBuffer<int8_t> d_red_spc, d_red_spl;

  // VTK output of a reference-order state (vtk.cpp); time series per output path
  void write_vtk(const std::vector<double>& x_ref, double t, const std::string& path, bool append) const;
  mutable std::map<std::string, std::vector<double>> vtk_steps;

  // host-side helpers
  std::vector<double> initial_state() const;        // reference DOF order
  void to_blocked(const std::vector<double>& ref, std::vector<double>& blk) const;
  void from_blocked(const std::vector<double>& blk, std::vector<double>& ref) const;
  int64_t ref_dof(int comp, int32_t vloc, int local) const;

  // assemble into r (residual, may be null) and J (BSR values, may be null):
  //   r += cm * M(x, t) + ca * A(x, t),  J += cm * dM/dx + ca * dA/dx
  // mode bit 1: residual, bit 2: Jacobian; with kAssembleOverwriteJacobian the Jacobian is
  // overwritten (J = cm dM/dx + ca dA/dx) instead of added to, and its prior contents are ignored.
  static constexpr int kAssembleOverwriteJacobian = 8;
  // kAssembleJacobianF32: the per-element Jacobian values of the state-dependent terms are
  // computed and gathered in fp32 (mixed precision; the residual and the static part stay fp64)
  static constexpr int kAssembleJacobianF32 = 16;
  // residual passes only: kAssembleStaticOnly adds the static part (cm Ms + ca Ks) x alone,
  // kAssembleDynamicOnly the state-dependent volume and face terms alone
  static constexpr int kAssembleStaticOnly = 32;
  static constexpr int kAssembleDynamicOnly = 64;
  // jac_sell32 (optional, sell_slots * 32 * bs * bs floats with zero padding slots): when one
  // volume gather produces every final Jacobian entry (one compartment, every slot
  // state-dependent, no membrane, padding or constraint rows), that gather also writes the
  // fp32 SELL-32 copy of J there; the return value says whether it did.
  bool assemble(const double* x, double t, double cm, double ca, double* r, double* J, int mode, cudaStream_t s,
                float* jac_sell32 = nullptr) const;
  // matrix-free Jacobian product y = (cm dM/dx + ca dA/dx)(x, t) v: the state-dependent
  // volume and face terms evaluated per element / face (mode kVolumeJacobianApply /
  // kFaceJacobianApply) and gathered like a residual, the constant terms from their matrices
  // assembled at set-up, unit rows for padded species slots and constrained DOFs
  void jacobian_apply(const double* x, double t, double cm, double ca, const double* v, double* y,
                      cudaStream_t s) const;
  Bsr bsr(double* val, float* val32) const;
  Sell sell() const;  // SELL-32 layout of the pattern (values sized sell_slots * 32 * bs * bs)
  int64_t sell_slots = 0;
  DeviceBuffer<int64_t> d_sell_off;
  DeviceBuffer<int32_t> d_sell_cols;
  DeviceBuffer<int64_t> d_sell_bpos;  // per BSR block: its SELL-32 value slot ((off + k) * 32 + lane)
  int64_t nnzb() const { return static_cast<int64_t>(colidx.size()); }

 private:
  void build_species();
  void build_nodes();
  void build_volume_groups();
  void build_face_groups();
  void build_pattern();
  void upload_geometry();
  void build_static_matrices();
  void build_constraints();
  void setup_volume_jit();
};

}  // namespace dcgpu
