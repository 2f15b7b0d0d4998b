// Volume kernels compiled at model set-up for one compartment's expression programs.
//
// The bytecode interpreter (interp.cuh) evaluates any program, but each bytecode
// instruction costs a dispatch and shared-memory register traffic; on GB300 the FP32
// Jacobian-only pass of the mixed-precision path is bound by that overhead rather than by
// arithmetic.  Here the compartment's residual and residual + Jacobian programs become
// straight-line CUDA code and its term lists compile-time tables of a Spec of the shared
// element body (volume_kernel.cuh); NVRTC compiles the kernels for sm_103a and they are
// launched in place of the interpreter's.  Compiled modules are cached per generated source
// for the life of the process.  NVRTC is loaded with dlopen: where it is missing or a
// compilation fails, the model keeps the interpreter kernels (also GPU code) and
// reports so.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "device.cuh"
#include "expr.hpp"

namespace dcgpu {

struct JitVolume {
  int dim = 0, ns = 0;
  // kernels: residual pass (mode 1), fp64 combined (mode 3), fp64 and fp32 Jacobian-only (mode 2)
  const void* k_res = nullptr;
  const void* k_both = nullptr;
  const void* k_jac64 = nullptr;
  const void* k_jac32 = nullptr;
  double compile_seconds = 0.0;
  int n_slots = 0;      // Jacobian slots of the element records (sizes the shared-memory staging)
  bool staged = false;  // element records staged in shared memory (vk::k_volume_jit)
};

// What the generator needs of one volume group (a compartment's cells).
struct JitVolumeInput {
  int dim = 0, ns = 0, species_offset = 0, n_slots = 0;
  bool all_mass = false;
  const Program* prog_res = nullptr;
  const Program* prog_all = nullptr;
  const std::vector<Term>* res_terms_r = nullptr;
  const std::vector<Term>* res_terms_a = nullptr;
  const std::vector<Term>* jac_terms = nullptr;
};

// CUDA source of the generated Specs and kernels (no compilation; for tests and logs).
std::string volume_jit_source(const JitVolumeInput& in);
// NVRTC compilation alone (no device needed): the cubin and the lowered kernel names of
// the four variants, or false with a message in *why.
bool compile_volume_jit(const JitVolumeInput& in, std::vector<char>* cubin, std::vector<std::string>* lowered,
                        std::string* why);
// Compiles (or takes from the cache) the kernels of one volume group; returns null with a
// message in *why when NVRTC is unavailable or the compilation fails.
std::shared_ptr<const JitVolume> build_volume_jit(const JitVolumeInput& in, std::string* why);
// One launch of a compiled kernel over cells [begin, end) (mode as launch_volume's).
void launch_volume_jit(const JitVolume& jit, const VolumeParams& p, int begin, int end, int mode,
                       cudaStream_t stream);

}  // namespace dcgpu
