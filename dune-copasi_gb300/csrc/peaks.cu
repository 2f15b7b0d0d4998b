// Arithmetic throughput of the device the library runs on (instrumentation): FP64 and FP32
// fused multiply-add rates, measured with independent FMA chains.  The volume assembly is
// bound by the FP64 pipe, whose rate on GB300 is a small fraction of the FP32 rate, so its
// roofline fraction is taken against this measured number.
#include <cuda_runtime.h>

#include "linalg.cuh"

namespace dcgpu {

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

// kChains independent chains x <- x a + b per thread; a < 1 keeps them bounded.  The sum
// is stored only under a condition that never holds, so the work cannot be removed.
template <class T>
__global__ void __launch_bounds__(kThreads) k_fma_rate(T* out, int iters, T a, T b) {
  T x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = static_cast<T>(threadIdx.x + c) * static_cast<T>(1e-3);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  T s = T(0);
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == static_cast<T>(-12345.0)) out[blockIdx.x * kThreads + threadIdx.x] = s;
}

template <class T>
double fma_rate(int iters) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
  const int blocks = sms * 8;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * kThreads) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const T a = static_cast<T>(0.999999), b = static_cast<T>(1e-6);
  k_fma_rate<T><<<blocks, kThreads>>>(out, iters, a, b);  // warm-up
  cudaEventRecord(e0);
  k_fma_rate<T><<<blocks, kThreads>>>(out, iters, a, b);
  cudaEventRecord(e1);
  count_launches(2);
  float ms = 0.0f;
  const bool ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
                  cudaGetLastError() == cudaSuccess;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (!ok || ms <= 0.0f) return -1.0;
  const double flops = 2.0 * kChains * static_cast<double>(iters) * blocks * kThreads;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

int fma_peaks(double* fp64_tflops, double* fp32_tflops) {
  const double d = fma_rate<double>(2048);
  const double f = fma_rate<float>(65536);
  if (d <= 0.0 || f <= 0.0) return 1;
  *fp64_tflops = d;
  *fp32_tflops = f;
  return 0;
}

}  // namespace dcgpu
