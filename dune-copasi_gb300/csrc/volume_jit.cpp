// Run-time compiled volume kernels (see volume_jit.hpp).
#include "volume_jit.hpp"

#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <type_traits>
#include <optional>

#include "linalg.cuh"
#include "model.hpp"
#include "volume_kernel.cuh"

// kJitHeaderNames / kJitHeaderSources: the text of device.cuh, bytecode.hpp, lookup.hpp and
// volume_kernel.cuh, embedded at build time
#include "jit_headers.inc"

namespace dcgpu {

namespace {

// <cstdint> as NVRTC sees it: the fixed-width types the shared headers use (same sizes as
// the host's, so VolumeParams has one layout on both sides)
const char* const kCstdintStub = R"DCSTUB(
#pragma once
typedef signed char int8_t;
typedef short int16_t;
typedef int int32_t;
typedef long long int64_t;
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
typedef unsigned long long uintptr_t;
namespace std {
using ::int8_t; using ::int16_t; using ::int32_t; using ::int64_t;
using ::uint8_t; using ::uint16_t; using ::uint32_t; using ::uint64_t; using ::uintptr_t;
}
)DCSTUB";

// ---------------------------------------------------------------------- NVRTC by dlopen
struct Nvrtc {
  bool ok = false;
  std::string why;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcAddNameExpression) add_name = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetLoweredName) lowered = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
};

const Nvrtc& nvrtc() {
  static const Nvrtc lib = [] {
    Nvrtc n;
    void* h = nullptr;
    for (const char* name : {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so"}) {
      h = dlopen(name, RTLD_NOW | RTLD_LOCAL);
      if (h) break;
    }
    if (!h) {
      n.why = "libnvrtc not found";
      return n;
    }
    auto sym = [&](auto& fn, const char* name) {
      fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(dlsym(h, name));
      if (!fn) n.why = std::string("libnvrtc lacks ") + name;
    };
    sym(n.create, "nvrtcCreateProgram");
    sym(n.add_name, "nvrtcAddNameExpression");
    sym(n.compile, "nvrtcCompileProgram");
    sym(n.log_size, "nvrtcGetProgramLogSize");
    sym(n.log, "nvrtcGetProgramLog");
    sym(n.lowered, "nvrtcGetLoweredName");
    sym(n.cubin_size, "nvrtcGetCUBINSize");
    sym(n.cubin, "nvrtcGetCUBIN");
    sym(n.destroy, "nvrtcDestroyProgram");
    n.ok = n.why.empty();
    return n;
  }();
  return lib;
}

// ---------------------------------------------------------------------- code generation
std::string dlit(double v) {
  // a double literal that reads back to the same bits (non-finite values by their bits)
  if (!std::isfinite(v)) {
    uint64_t bits;
    std::memcpy(&bits, &v, sizeof bits);
    char buf[64];
    std::snprintf(buf, sizeof buf, "__longlong_as_double(0x%016llxLL)", static_cast<unsigned long long>(bits));
    return buf;
  }
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.17g", v);
  std::string s = buf;
  if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
  return "(" + s + ")";
}

std::string term_init(const Term& t) {
  std::ostringstream o;
  o << "Term{" << int(t.kind) << ", " << int(t.form) << ", " << int(t.test) << ", " << int(t.trial) << ", "
    << int(t.side) << ", " << int(t.slot) << ", " << t.out << ", " << t.coef << ", 0}";
  return o.str();
}

// value of program input `id` in the element body's names (the mapping of vk::volume_input)
std::string input_expr(uint16_t id, int dim, int ns, int soff) {
  if (id < IN_GRAD) {
    const int s = static_cast<int>(id) - soff;
    return (s >= 0 && s < ns) ? "u[" + std::to_string(s) + "]" : "F(0)";
  }
  if (id < IN_POSITION) {
    const int gi = static_cast<int>(id) - IN_GRAD;
    const int s = gi / 3 - soff, ax = gi % 3;
    return (s >= 0 && s < ns && ax < dim) ? "g[" + std::to_string(s) + "][" + std::to_string(ax) + "]" : "F(0)";
  }
  if (id < IN_NORMAL) {
    const int ax = static_cast<int>(id) - IN_POSITION;
    return ax < dim ? "xq[" + std::to_string(ax) + "]" : "F(0)";
  }
  switch (id) {
    case IN_TIME: return "t";
    case IN_ENTITY_VOLUME: return "vol";
    case IN_IN_VOLUME: return "F(1)";
    default: return "F(0)";
  }
}

// the program as straight-line statements over R[] (the operations of interp.cuh's apply_op,
// in the same order)
std::string program_code(const Program& p, int dim, int ns, int soff) {
  std::ostringstream o;
  for (size_t i = 0; i < p.inputs.size(); ++i) o << "    R[" << i << "] = " << input_expr(p.inputs[i], dim, ns, soff) << ";\n";
  for (const Instr& ins : p.code) {
    const std::string A = "R[" + std::to_string(ins.a) + "]", B = "R[" + std::to_string(ins.b) + "]",
                      C = "R[" + std::to_string(ins.c) + "]";
    std::string v;
    auto f1 = [&](const char* fn) { return std::string(fn) + "(" + A + ")"; };
    auto f2 = [&](const char* fn) { return std::string(fn) + "(" + A + ", " + B + ")"; };
    auto cmp = [&](const char* op) { return "(" + A + " " + op + " " + B + " ? F(1) : F(0))"; };
    switch (ins.op) {
      case OP_CONST: v = "static_cast<F>" + dlit(p.consts[ins.a | (ins.b << 8)]); break;
      case OP_ADD: v = A + " + " + B; break;
      case OP_SUB: v = A + " - " + B; break;
      case OP_MUL: v = A + " * " + B; break;
      case OP_DIV: v = A + " / " + B; break;
      case OP_POW: v = f2("pow"); break;
      case OP_FMOD: v = f2("fmod"); break;
      case OP_ATAN2: v = f2("atan2"); break;
      case OP_HYPOT: v = f2("hypot"); break;
      case OP_MIN: v = f2("fmin"); break;
      case OP_MAX: v = f2("fmax"); break;
      case OP_LT: v = cmp("<"); break;
      case OP_LE: v = cmp("<="); break;
      case OP_GT: v = cmp(">"); break;
      case OP_GE: v = cmp(">="); break;
      case OP_EQ: v = cmp("=="); break;
      case OP_NE: v = cmp("!="); break;
      case OP_AND: v = "((" + A + " != F(0) && " + B + " != F(0)) ? F(1) : F(0))"; break;
      case OP_OR: v = "((" + A + " != F(0) || " + B + " != F(0)) ? F(1) : F(0))"; break;
      case OP_NEG: v = "-" + A; break;
      case OP_NOT: v = "(" + A + " != F(0) ? F(0) : F(1))"; break;
      case OP_SQR: v = A + " * " + A; break;
      case OP_CUBE: v = A + " * " + A + " * " + A; break;
      case OP_RECIP: v = "F(1) / " + A; break;
      case OP_EXP: v = f1("exp"); break;
      case OP_LOG: v = f1("log"); break;
      case OP_LOG2: v = f1("log2"); break;
      case OP_LOG10: v = f1("log10"); break;
      case OP_SQRT: v = f1("sqrt"); break;
      case OP_SIN: v = f1("sin"); break;
      case OP_COS: v = f1("cos"); break;
      case OP_TAN: v = f1("tan"); break;
      case OP_ASIN: v = f1("asin"); break;
      case OP_ACOS: v = f1("acos"); break;
      case OP_ATAN: v = f1("atan"); break;
      case OP_SINH: v = f1("sinh"); break;
      case OP_COSH: v = f1("cosh"); break;
      case OP_TANH: v = f1("tanh"); break;
      case OP_ASINH: v = f1("asinh"); break;
      case OP_ACOSH: v = f1("acosh"); break;
      case OP_ATANH: v = f1("atanh"); break;
      case OP_ABS: v = f1("fabs"); break;
      case OP_SIGN: v = "(" + A + " < F(0) ? -F(1) : (" + A + " > F(0) ? F(1) : F(0)))"; break;
      case OP_RINT: v = f1("rint"); break;
      case OP_FLOOR: v = f1("floor"); break;
      case OP_CEIL: v = f1("ceil"); break;
      case OP_ROUND: v = f1("round"); break;
      case OP_TRUNC: v = f1("trunc"); break;
      case OP_ERF: v = f1("erf"); break;
      case OP_ERFC: v = f1("erfc"); break;
      case OP_SEL: v = "(" + A + " != F(0) ? " + B + " : " + C + ")"; break;
      case OP_POWI: {
        // binary exponentiation with the interpreter's order of multiplications
        const int e = static_cast<int8_t>(ins.c);
        int n = e < 0 ? -e : e;
        o << "    { F r_ = F(1), x_ = " << A << ";\n";
        while (n) {
          if (n & 1) o << "      r_ *= x_;\n";
          o << "      x_ *= x_;\n";
          n >>= 1;
        }
        o << "      R[" << int(ins.dst) << "] = " << (e < 0 ? "F(1) / r_" : "r_") << "; }\n";
        continue;
      }
      case OP_INTERP:
        v = "static_cast<F>(interp_lookup(P.tables.x + P.tables.off[" + std::to_string(ins.b) + "], P.tables.y + "
            "P.tables.off[" + std::to_string(ins.b) + "], P.tables.len[" + std::to_string(ins.b) +
            "], static_cast<double>(" + A + ")))";
        break;
      case OP_FTAB:
        v = "static_cast<F>(ftab_lookup(P.tables.ft[" + std::to_string(ins.b) + "], P.tables.ftg, static_cast<double>(" +
            A + ")))";
        break;
      case OP_TIFF:
        v = "static_cast<F>(image_lookup(P.tables.im[" + std::to_string(ins.b) +
            "], P.tables.imp, static_cast<double>(" + A + "), static_cast<double>(" + C + ")))";
        break;
      default: v = "static_cast<F>(__longlong_as_double(0x7ff8000000000000LL))"; break;
    }
    o << "    R[" << int(ins.dst) << "] = " << v << ";\n";
  }
  return o.str();
}

int coef_count(const std::vector<Term>& jac, int dim) {
  const int nq = dim == 2 ? 3 : 4;
  int n = 0;
  for (const Term& T : jac) {
    const int sz = (T.kind == J_MASS || T.kind == J_MASS_U || T.kind == J_STORAGE_SELF) ? nq + 1
                   : T.kind == J_DIFF_SCALAR                                             ? 1
                   : T.kind == J_DIFF_TENSOR                                             ? dim * dim
                                                                                         : (dim + 1) * dim;
    n = std::max(n, static_cast<int>(T.coef) + sz);
  }
  return n;
}

// one generated Spec: a program with its residual and Jacobian term lists
// whether the kernels stage their element records in shared memory (all four variants)
bool jit_stages(const JitVolumeInput& in) {
  return vk::jit_stage_bytes(in.dim, in.ns, in.n_slots, 3, 8) <= vk::kJitStageMax;
}

std::string spec_code(const char* name, const Program& prog, const std::vector<Term>& res,
                      const std::vector<Term>& jac, const JitVolumeInput& in) {
  VolumeParams flags{};
  set_volume_flags(flags, prog, res, jac, in.dim);
  const int ncoef = coef_count(jac, in.dim);
  std::ostringstream o;
  o << "struct " << name << " {\n"
    << "  static constexpr bool kUnrollPoints = true;\n"
    << "  static constexpr int kRegs = " << std::max(prog.nregs, 1) << ";\n"
    << "  static constexpr int kCoefs = " << std::max(ncoef, 1) << ";\n"
    << "  static constexpr int kSlots = " << in.n_slots << ";\n"
    << "  static constexpr bool kStage = " << (jit_stages(in) ? "true" : "false") << ";\n"
    << "  __device__ __forceinline__ static constexpr int n_res(const VolumeParams&, bool) { return " << res.size()
    << "; }\n"
    << "  __device__ __forceinline__ static constexpr Term res(const VolumeParams&, bool, int t) {\n"
    << "    switch (t) {\n";
  for (size_t i = 0; i < res.size(); ++i) o << "      case " << i << ": return " << term_init(res[i]) << ";\n";
  o << "      default: return Term{};\n    }\n  }\n"
    << "  __device__ __forceinline__ static constexpr int n_jac(const VolumeParams&) { return " << jac.size() << "; }\n"
    << "  __device__ __forceinline__ static constexpr Term jac(const VolumeParams&, int t) {\n"
    << "    switch (t) {\n";
  for (size_t i = 0; i < jac.size(); ++i) o << "      case " << i << ": return " << term_init(jac[i]) << ";\n";
  o << "      default: return Term{};\n    }\n  }\n"
    << "  __device__ __forceinline__ static constexpr int out(const VolumeParams&, bool, int i) {\n"
    << "    switch (i) {\n";
  for (size_t i = 0; i < prog.outputs.size(); ++i) o << "      case " << i << ": return " << int(prog.outputs[i]) << ";\n";
  o << "      default: return 0;\n    }\n  }\n"
    << "  __device__ __forceinline__ static constexpr int n_slots(const VolumeParams&) { return " << in.n_slots
    << "; }\n"
    << "  __device__ __forceinline__ static constexpr bool all_mass(const VolumeParams&) { return "
    << (in.all_mass ? "true" : "false") << "; }\n"
    << "  __device__ __forceinline__ static constexpr bool need_grad(const VolumeParams&) { return "
    << (flags.need_grad ? "true" : "false") << "; }\n"
    << "  __device__ __forceinline__ static constexpr bool has_flux(const VolumeParams&) { return "
    << (flags.has_flux ? "true" : "false") << "; }\n"
    << "  __device__ __forceinline__ static constexpr bool need_pos(const VolumeParams&) { return "
    << (flags.need_pos ? "true" : "false") << "; }\n"
    << "  __device__ __forceinline__ static constexpr bool need_vol(const VolumeParams&) { return "
    << (flags.need_vol ? "true" : "false") << "; }\n"
    << "  __device__ __forceinline__ static constexpr int coef_bound(const VolumeParams&, int) { return " << ncoef
    << "; }\n"
    << "  template <class F>\n"
    << "  __device__ __forceinline__ static ArrCast<F> as_float(const Arr<F>& c) { return ArrCast<F>{c.p}; }\n"
    << "  template <int DIM, int NS, class F, class Regs>\n"
    << "  __device__ __forceinline__ static void run(const VolumeParams& P, bool, Regs R, const F (&u)[NS],\n"
    << "                                             const F (&g)[NS][DIM], const F (&xq)[DIM], F t, F vol) {\n"
    << "    (void)P; (void)u; (void)g; (void)xq; (void)t; (void)vol;\n"
    << program_code(prog, in.dim, in.ns, in.species_offset) << "  }\n};\n";
  return o.str();
}

const char* const kVariantNames[4] = {"k_res", "k_both", "k_jac64", "k_jac32"};

std::string kernel_name(const JitVolumeInput& in, int variant) {
  const std::string dn = std::to_string(in.dim) + ", " + std::to_string(in.ns);
  switch (variant) {
    case 0: return "dcgpu::vk::k_volume_jit<" + dn + ", double, dcgpu::jitgen::SpecRes, 1>";
    case 1: return "dcgpu::vk::k_volume_jit<" + dn + ", double, dcgpu::jitgen::SpecAll, 3>";
    case 2: return "dcgpu::vk::k_volume_jit<" + dn + ", double, dcgpu::jitgen::SpecAll, 2>";
    default: return "dcgpu::vk::k_volume_jit<" + dn + ", float, dcgpu::jitgen::SpecAll, 2>";
  }
}

struct CacheEntry {
  std::shared_ptr<JitVolume> jit;
  cudaLibrary_t lib = nullptr;
};

std::mutex g_cache_mutex;
std::map<std::string, CacheEntry> g_cache;

}  // namespace

std::string volume_jit_source(const JitVolumeInput& in) {
  std::ostringstream o;
  o << "// generated: volume kernels of one compartment (dim " << in.dim << ", " << in.ns << " species)\n"
    << "#include \"volume_kernel.cuh\"\n"
    << "namespace dcgpu {\nnamespace jitgen {\nusing namespace dcgpu::vk;\n"
    << spec_code("SpecRes", *in.prog_res, *in.res_terms_r, {}, in)
    << spec_code("SpecAll", *in.prog_all, *in.res_terms_a, *in.jac_terms, in) << "}  // namespace jitgen\n}  // namespace dcgpu\n";
  return o.str();
}

bool compile_volume_jit(const JitVolumeInput& in, std::vector<char>* cubin_out, std::vector<std::string>* lowered_out,
                        std::string* why) {
  const std::string src = volume_jit_source(in);
  const Nvrtc& nv = nvrtc();
  if (!nv.ok) {
    if (why) *why = nv.why;
    return false;
  }
  std::vector<const char*> hdr_src, hdr_names;
  for (size_t i = 0; i < sizeof(kJitHeaderNames) / sizeof(kJitHeaderNames[0]); ++i) {
    hdr_names.push_back(kJitHeaderNames[i]);
    hdr_src.push_back(kJitHeaderSources[i]);
  }
  hdr_names.push_back("cstdint");
  hdr_src.push_back(kCstdintStub);
  nvrtcProgram prog = nullptr;
  if (nv.create(&prog, src.c_str(), "dcgpu_volume_jit.cu", static_cast<int>(hdr_src.size()), hdr_src.data(),
                hdr_names.data()) != NVRTC_SUCCESS) {
    if (why) *why = "nvrtcCreateProgram failed";
    return false;
  }
  std::string names[4];
  for (int v = 0; v < 4; ++v) {
    names[v] = kernel_name(in, v);
    nv.add_name(prog, names[v].c_str());
  }
  // DCGPU_JIT_VERBOSE=1: ptxas resource usage of the compiled kernels on stderr
  const bool verbose = std::getenv("DCGPU_JIT_VERBOSE") != nullptr;
  const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-DNDEBUG", "--ptxas-options=-v"};
  const nvrtcResult cr = nv.compile(prog, verbose ? 4 : 3, opts);
  if (verbose && cr == NVRTC_SUCCESS) {
    size_t n = 0;
    nv.log_size(prog, &n);
    std::string log(n, '\0');
    if (n) nv.log(prog, &log[0]);
    std::fprintf(stderr, "%s\n", log.c_str());
  }
  if (cr != NVRTC_SUCCESS) {
    size_t n = 0;
    nv.log_size(prog, &n);
    std::string log(n, '\0');
    if (n) nv.log(prog, &log[0]);
    if (why) *why = "NVRTC compilation failed: " + log.substr(0, 4000);
    nv.destroy(&prog);
    return false;
  }
  size_t nbin = 0;
  nv.cubin_size(prog, &nbin);
  cubin_out->assign(nbin, 0);
  nv.cubin(prog, cubin_out->data());
  lowered_out->assign(4, std::string());
  for (int v = 0; v < 4; ++v) {
    const char* ln = nullptr;
    if (nv.lowered(prog, names[v].c_str(), &ln) != NVRTC_SUCCESS || !ln) {
      if (why) *why = "nvrtcGetLoweredName failed for " + names[v];
      nv.destroy(&prog);
      return false;
    }
    (*lowered_out)[v] = ln;
  }
  nv.destroy(&prog);
  return true;
}

std::shared_ptr<const JitVolume> build_volume_jit(const JitVolumeInput& in, std::string* why) {
  const std::string src = volume_jit_source(in);
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  auto it = g_cache.find(src);
  if (it != g_cache.end()) return it->second.jit;
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<char> cubin;
  std::vector<std::string> lowered;
  if (!compile_volume_jit(in, &cubin, &lowered, why)) return nullptr;
  CacheEntry e;
  if (cudaLibraryLoadData(&e.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess) {
    (void)cudaGetLastError();
    if (why) *why = "cudaLibraryLoadData failed";
    return nullptr;
  }
  auto jit = std::make_shared<JitVolume>();
  jit->dim = in.dim;
  jit->ns = in.ns;
  const void** slots[4] = {&jit->k_res, &jit->k_both, &jit->k_jac64, &jit->k_jac32};
  for (int v = 0; v < 4; ++v) {
    cudaKernel_t k = nullptr;
    if (cudaLibraryGetKernel(&k, e.lib, lowered[v].c_str()) != cudaSuccess || !k) {
      (void)cudaGetLastError();
      if (why) *why = std::string("cudaLibraryGetKernel failed for ") + kVariantNames[v];
      return nullptr;
    }
    *slots[v] = reinterpret_cast<const void*>(k);
    // the staging area of the largest variant (fp64 residual and Jacobian records)
    const int need = jit_stages(in) ? vk::jit_stage_bytes(in.dim, in.ns, in.n_slots, 3, 8) : 0;
    if (need > 48 * 1024 &&
        cudaFuncSetAttribute(*slots[v], cudaFuncAttributeMaxDynamicSharedMemorySize, need) != cudaSuccess) {
      (void)cudaGetLastError();
      if (why) *why = "cannot raise the shared-memory limit of the compiled volume kernels";
      return nullptr;
    }
  }
  jit->n_slots = in.n_slots;
  jit->staged = jit_stages(in);
  jit->compile_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  e.jit = jit;
  g_cache.emplace(src, e);
  return jit;
}

void launch_volume_jit(const JitVolume& jit, const VolumeParams& p, int begin, int end, int mode,
                       cudaStream_t stream) {
  const int n = end - begin;
  if (n <= 0) return;
  if (mode == 3 && p.jac_f32) {
    // residual in fp64 and the element Jacobian in fp32 (mixed precision): two passes, the
    // second entirely in fp32, cost less than one pass that forms the Jacobian coefficients
    // in fp64 on GB300's narrow FP64 pipe
    launch_volume_jit(jit, p, begin, end, 1, stream);
    launch_volume_jit(jit, p, begin, end, 2, stream);
    return;
  }
  const void* k = nullptr;
  if (mode == 1) k = jit.k_res;
  else if (mode == 3) k = jit.k_both;
  else if (mode == 2) k = p.jac_f32 ? jit.k_jac32 : jit.k_jac64;
  if (!k) throw std::runtime_error("run-time compiled volume kernel: unsupported mode " + std::to_string(mode));
  // element values of the staged Jacobian records: fp64 unless the pass runs in fp32 or rounds to it
  const bool ej64 = (mode == 2 && k == jit.k_jac64) || (mode == 3 && !p.jac_f32);
  const int smem = jit.staged ? vk::jit_stage_bytes(jit.dim, jit.ns, jit.n_slots, mode, ej64 ? 8 : 4) : 0;
  VolumeParams pp = p;
  int b = begin, e = end;
  void* args[] = {&pp, &b, &e};
  count_launches(1);
  constexpr int kThreads = vk::kJitThreads;
  const cudaError_t err =
      cudaLaunchKernel(k, dim3((n + kThreads - 1) / kThreads), dim3(kThreads), args, smem, stream);
  if (err != cudaSuccess) throw CudaError(std::string("run-time compiled volume kernel: ") + cudaGetErrorString(err));
}

// ---------------------------------------------------------------------- self-test
namespace {

// A synthetic two-species compartment whose terms cover every volume term kind, compiled
// for DIM (no device needed)
bool selftest_dim(int dim, std::string* why, double* seconds) {
  ParserContext ctx;
  ctx.constants["F"] = 0.04;
  Resolver res = [](const std::string& nm) -> std::optional<Symbol> {
    Symbol s;
    s.is_input = true;
    if (nm == "u") s.input = IN_SPECIES + 0;
    else if (nm == "v") s.input = IN_SPECIES + 1;
    else if (nm == "grad_u_x") s.input = IN_GRAD + 0;
    else if (nm == "position_x") s.input = IN_POSITION + 0;
    else if (nm == "entity_volume") s.input = IN_ENTITY_VOLUME;
    else if (nm == "time") s.input = IN_TIME;
    else return std::nullopt;
    return s;
  };
  const char* exprs[] = {
      "-u*v^2 + F*(1-u)",                 // 0 reaction u
      "u*v^2 - (F+0.06)*v",               // 1 reaction v
      "-v^2 - F",                         // 2 d/du reaction u
      "-2*u*v",                           // 3 d/dv reaction u
      "0.1*position_x + time",            // 4.. velocity of u
      "0.2*sin(position_x)",
      "0",
      "1e-3*(1 + grad_u_x^2)",            // 7 diffusion of u by v
      "1 + 0.5*u",                        // 8 storage of v
      "1e-2", "1e-3", "-1e-3", "2e-2",    // 9.. tensor diffusion of v (up to 3x3)
      "1e-4", "0", "0", "0", "3e-2",
      "2e-3*grad_u_x",                    // 18 d/d grad: non-linear diffusion Jacobian
      "entity_volume > 0 ? exp(-u) : log(1+v)",  // 19 extra reaction-like term
  };
  ProgramBuilder b(ctx);
  for (const char* e : exprs) b.add_output(b.compile_text(e, res));
  const Program prog = b.finish();
  const int nq = dim == 2 ? 3 : 4;
  auto T = [](uint8_t kind, uint8_t form, uint8_t test, uint8_t trial, uint8_t slot, uint16_t out, uint16_t coef) {
    Term t{};
    t.kind = kind;
    t.form = form;
    t.test = test;
    t.trial = trial;
    t.slot = slot;
    t.out = out;
    t.coef = coef;
    return t;
  };
  std::vector<Term> rterms = {T(R_REACTION, 1, 0, 0, 0, 0, 0), T(R_REACTION, 1, 1, 1, 0, 1, 0),
                              T(R_VELOCITY, 1, 0, 0, 0, 4, 0), T(R_DIFF_SCALAR, 1, 0, 1, 0, 7, 0),
                              T(R_STORAGE, 0, 1, 1, 0, 8, 0), T(R_DIFF_TENSOR, 1, 1, 1, 0, 9, 0),
                              T(R_REACTION, 1, 1, 1, 0, 19, 0)};
  int c = 0;
  std::vector<Term> jterms;
  auto add = [&](uint8_t kind, uint8_t form, uint8_t test, uint8_t trial, uint8_t slot, uint16_t out, int size) {
    jterms.push_back(T(kind, form, test, trial, slot, out, static_cast<uint16_t>(c)));
    c += size;
  };
  add(J_MASS, 1, 0, 0, 0, 2, nq + 1);
  add(J_VELOCITY, 1, 0, 0, 0, 4, (dim + 1) * dim);
  add(J_MASS, 1, 0, 1, 1, 3, nq + 1);
  add(J_DIFF_SCALAR, 1, 0, 1, 1, 7, 1);
  add(J_DIFFJAC_SCALAR, 1, 0, 0, 0 + 2, 18, (dim + 1) * dim);
  add(J_STORAGE_SELF, 0, 1, 1, 3, 8, nq + 1);
  add(J_MASS_U, 0, 1, 0, 4, 8, nq + 1);
  add(J_DIFF_TENSOR, 1, 1, 1, 3, 9, dim * dim);
  add(J_VELOCITY_JAC, 1, 0, 1, 1, 4, (dim + 1) * dim);
  // slots must be ascending in the list
  std::stable_sort(jterms.begin(), jterms.end(), [](const Term& a, const Term& b) { return a.slot < b.slot; });
  JitVolumeInput in;
  in.dim = dim;
  in.ns = 2;
  in.species_offset = 0;
  in.n_slots = 5;
  in.all_mass = false;
  in.prog_res = &prog;
  in.prog_all = &prog;
  in.res_terms_r = &rterms;
  in.res_terms_a = &rterms;
  in.jac_terms = &jterms;
  std::vector<char> cubin;
  std::vector<std::string> lowered;
  const auto t0 = std::chrono::steady_clock::now();
  const bool ok = compile_volume_jit(in, &cubin, &lowered, why);
  *seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return ok && !cubin.empty();
}

}  // namespace

}  // namespace dcgpu

extern "C" int dc_jit_selftest(char* message, size_t len) {
  std::string why;
  double seconds = 0.0;
  bool ok = false;
  try {
    ok = dcgpu::selftest_dim(2, &why, &seconds) && dcgpu::selftest_dim(3, &why, &seconds);
  } catch (const std::exception& e) {
    why = e.what();
  }
  const std::string msg = ok ? "compiled 2 x 4 kernels in " + std::to_string(seconds) + " s" : why;
  if (message && len) {
    std::strncpy(message, msg.c_str(), len - 1);
    message[len - 1] = '\0';
  }
  return ok ? 0 : 4;
}
