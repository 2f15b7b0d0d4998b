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
// Set-up: the first call on a device, made with that device current, looks up the
// array's device address with cudaGetSymbolAddress.  Make that first call before any
// stream capture.
#include <mutex>

#include "../../include/dcgpu.h"
#include "handle.hpp"

namespace {

constexpr int64_t kNoAllocMaxDof = int64_t{1} << 20;
constexpr int kMaxDevices = 64;

// [0, kNoAllocMaxDof): staged state; [kNoAllocMaxDof, 2 kNoAllocMaxDof): residual
static __device__ __align__(256) double g_noalloc_stage[2 * kNoAllocMaxDof];

// device address of the array, looked up once per device with that device current; host
// code must not pass g_noalloc_stage itself to a kernel (it is a host-side stand-in)
double* g_stage_ptr[kMaxDevices] = {nullptr};
cudaError_t g_stage_err[kMaxDevices] = {cudaSuccess};
std::once_flag g_stage_once[kMaxDevices];

}  // namespace

extern "C" int dc_assemble_residual_noalloc(dc_model* handle, const double* x, double t, double cm,
                                            double ca, double* r) {
  if (!handle || !x || !r || !handle->model) return DC_ERR_ARGUMENT;
  const dcgpu::Model& m = *handle->model;
  // the staged layout is the reference DOF order, which the device layout equals unless
  // compartments carry different species counts (padded block rows)
  if (m.padded) return DC_ERR_ARGUMENT;
  const int64_t n = m.nnodes * m.bs;
  if (n > kNoAllocMaxDof) return DC_ERR_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DC_ERR_CUDA;
  std::call_once(g_stage_once[dev], [dev] {
    void* p = nullptr;
    g_stage_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_stage);
    g_stage_ptr[dev] = static_cast<double*>(p);
  });
  if (g_stage_err[dev] != cudaSuccess || g_stage_ptr[dev] == nullptr) return DC_ERR_CUDA;
  double* xs = g_stage_ptr[dev];
  double* rs = g_stage_ptr[dev] + kNoAllocMaxDof;
  cudaStream_t s = handle->stream;
  if (cudaMemcpyAsync(xs, x, n * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess) return DC_ERR_CUDA;
  if (cudaMemsetAsync(rs, 0, n * sizeof(double), s) != cudaSuccess) return DC_ERR_CUDA;
  try {
    m.assemble(xs, t, cm, ca, rs, nullptr, 1, s);
  } catch (...) {
    return DC_ERR_INTERNAL;
  }
  if (cudaMemcpyAsync(r, rs, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return DC_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return DC_ERR_CUDA;
  if (cudaGetLastError() != cudaSuccess) return DC_ERR_CUDA;
  return DC_OK;
}
