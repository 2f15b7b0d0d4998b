// Residual assembly that allocates no memory (dc_assemble_residual_noalloc).
//
// Some callers cannot allocate device memory at the moment they need a residual: a
// serving process whose device memory is already owned by another allocator (a
// framework's caching pool, a fixed per-tenant budget), or a latency-bound loop that must
// not call cudaMalloc/cudaFree because those calls can synchronise the whole device and
// stall every other stream.  dc_assemble stages the state and the residual in device
// buffers that it allocates on first use; this entry point stages them in one fixed
// array compiled into the library instead, so a call allocates nothing on the device or
// on the host.
//
// Limit: the array holds kNoAllocMaxDof (2^20) state values and as many residual values,
// 16 MiB in total, and every GPU that loads the library keeps it until the process
// exits.  All calls on one device share it.  Each call clears the residual half before
// assembling into it and overwrites the state half, so a call never sees the previous
// call's data; but calls whose work overlaps on the GPU (several host threads, or several
// models on one device) race on the array, and the caller must serialise them.
//
// Set-up: model creation (dc_model_create) looks up the array's device address on the
// model's device with cudaGetSymbolAddress.  That lookup is what loads the library module
// holding the array and commits its 16 MiB, so it happens where the caller allocates
// anyway.  If it failed there, the first call on that device retries it, and a call then
// may load the module: create the model, or make one call, before any stream capture.
// Only a successful lookup is kept.
#include <mutex>

#include "../../include/dcgpu.h"
#include "handle.hpp"

namespace {

constexpr int64_t kNoAllocMaxDof = int64_t{1} << 20;
constexpr int kMaxDevices = 64;

// [0, kNoAllocMaxDof): staged state; [kNoAllocMaxDof, 2 kNoAllocMaxDof): residual
static __device__ __align__(256) double g_noalloc_stage[2 * kNoAllocMaxDof];

// device address of the array per device, looked up with that device current; host code
// must not pass g_noalloc_stage itself to a kernel (it is a host-side stand-in)
std::mutex g_stage_mutex;
double* g_stage_ptr[kMaxDevices] = {nullptr};

// the array's address on `dev`, which must be the current device; nullptr if the lookup fails
double* stage_address(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_stage_mutex);
  if (!g_stage_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_stage) != cudaSuccess) {
      (void)cudaGetLastError();  // clear this thread's record of the failed lookup
      return nullptr;
    }
    g_stage_ptr[dev] = static_cast<double*>(p);
  }
  return g_stage_ptr[dev];
}

// the work of one call, with the model's device current
int residual_on_device(dc_model* handle, const double* x, double t, double cm, double ca, double* r, int64_t n) {
  double* stage = stage_address(handle->device);
  if (!stage) return DC_ERR_CUDA;
  double* xs = stage;
  double* rs = stage + kNoAllocMaxDof;
  cudaStream_t s = handle->stream;
  if (cudaMemcpyAsync(xs, x, n * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess) return DC_ERR_CUDA;
  if (cudaMemsetAsync(rs, 0, n * sizeof(double), s) != cudaSuccess) return DC_ERR_CUDA;
  try {
    handle->model->assemble(xs, t, cm, ca, rs, nullptr, 1, s);
  } catch (const dcgpu::CudaError&) {
    return DC_ERR_CUDA;
  } catch (...) {
    return DC_ERR_INTERNAL;
  }
  if (cudaMemcpyAsync(r, rs, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return DC_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return DC_ERR_CUDA;
  return DC_OK;
}

}  // namespace

bool dc_noalloc_prepare(int device) {
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) return false;
  if (cur != device && cudaSetDevice(device) != cudaSuccess) return false;
  const bool ok = stage_address(device) != nullptr;
  if (cur != device) cudaSetDevice(cur);
  return ok;
}

extern "C" int dc_assemble_residual_noalloc(dc_model* handle, const double* x, double t, double cm,
                                            double ca, double* r) {
  if (!handle || !x || !r || !handle->model) return DC_ERR_ARGUMENT;
  const dcgpu::Model& m = *handle->model;
  // the staged layout is the reference DOF order, which the device layout equals unless
  // compartments carry different species counts (padded block rows)
  if (m.padded) return DC_ERR_ARGUMENT;
  const int64_t n = m.nnodes * m.bs;
  if (n > kNoAllocMaxDof) return DC_ERR_ARGUMENT;
  // the array is looked up, and the work launched, on the device the model lives on,
  // whatever device the calling thread has current
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) return DC_ERR_CUDA;
  if (cur != handle->device && cudaSetDevice(handle->device) != cudaSuccess) return DC_ERR_CUDA;
  const int st = residual_on_device(handle, x, t, cm, ca, r, n);
  if (cur != handle->device && cudaSetDevice(cur) != cudaSuccess) return DC_ERR_CUDA;
  return st;
}
