// Vector kernels of the restarted GMRES solver (dune-istl RestartedGMResSolver, registered
// as "RestartedGMRes" in solver/istl/factory/iterative.hh:95-96, restart default 40).  The
// Krylov basis V is stored as (m+1) contiguous vectors of length n; the Hessenberg
// coefficients live on the device and are read by the host once per iteration for the Givens
// rotations.  Dot products are deterministic (fixed block partition, fixed final order).
#include "gmres.cuh"

#include <stdexcept>

#include "linalg.cuh"

namespace dcgpu {

namespace {

constexpr int kThreads = 256;

// partial[b * k + i] = sum over block b's slice of V_i . w, i < k
template <class T>
__global__ void __launch_bounds__(kThreads) k_mdot_partial(const T* __restrict__ V, int64_t n, int k,
                                                           const T* __restrict__ w, double* __restrict__ partial) {
  __shared__ double sh[kThreads];
  for (int i = 0; i < k; ++i) {
    const T* vi = V + static_cast<int64_t>(i) * n;
    double acc = 0.0;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x)
      acc += static_cast<double>(vi[t]) * static_cast<double>(w[t]);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[static_cast<int64_t>(blockIdx.x) * k + i] = sh[0];
    __syncthreads();
  }
}

// out[i] (+)= sum over blocks of partial[b * k + i], in block order
__global__ void k_mdot_final(const double* __restrict__ partial, int nblocks, int k, double* __restrict__ out,
                             int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  double acc = 0.0;
  for (int b = 0; b < nblocks; ++b) acc += partial[static_cast<int64_t>(b) * k + i];
  out[i] = accumulate ? out[i] + acc : acc;
}

// w += sign * sum_i h[i] V_i
template <class T>
__global__ void __launch_bounds__(kThreads) k_maxpy(T* __restrict__ w, const T* __restrict__ V, int64_t n, int k,
                                                    const double* __restrict__ h, double sign) {
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double acc = 0.0;
    for (int i = 0; i < k; ++i) acc += h[i] * static_cast<double>(V[static_cast<int64_t>(i) * n + t]);
    w[t] = static_cast<T>(static_cast<double>(w[t]) + sign * acc);
  }
}

// y = x / s[0]
template <class T>
__global__ void k_scale_by(T* __restrict__ y, const T* __restrict__ x, int64_t n, const double* __restrict__ s) {
  const double inv = 1.0 / s[0];
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x)
    y[t] = static_cast<T>(static_cast<double>(x[t]) * inv);
}

// y = a * x  (a by value)
template <class T>
__global__ void k_scale_value(T* __restrict__ y, const T* __restrict__ x, int64_t n, double a) {
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x)
    y[t] = static_cast<T>(a * static_cast<double>(x[t]));
}

// y = b - y
template <class T>
__global__ void k_sub_from(T* __restrict__ y, const T* __restrict__ b, int64_t n) {
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x)
    y[t] = b[t] - y[t];
}

int grid_of(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b > kGmresBlocks) b = kGmresBlocks;
  return static_cast<int>(b < 1 ? 1 : b);
}

}  // namespace

template <class T>
void gmres_mdot(const T* V, int64_t n, int k, const T* w, double* out, double* partial, bool accumulate,
                cudaStream_t s) {
  if (k <= 0) return;
  const int nb = grid_of(n);
  count_launches(2);
  k_mdot_partial<T><<<nb, kThreads, 0, s>>>(V, n, k, w, partial);
  k_mdot_final<<<(k + 63) / 64, 64, 0, s>>>(partial, nb, k, out, accumulate ? 1 : 0);
}

template <class T>
void gmres_maxpy(T* w, const T* V, int64_t n, int k, const double* h, double sign, cudaStream_t s) {
  if (k <= 0 || n == 0) return;
  count_launches(1);
  k_maxpy<T><<<grid_of(n), kThreads, 0, s>>>(w, V, n, k, h, sign);
}

template <class T>
void gmres_scale(T* y, const T* x, int64_t n, const double* by, cudaStream_t s) {
  if (n == 0) return;
  count_launches(1);
  k_scale_by<T><<<grid_of(n), kThreads, 0, s>>>(y, x, n, by);
}

template <class T>
void gmres_scale_value(T* y, const T* x, int64_t n, double a, cudaStream_t s) {
  if (n == 0) return;
  count_launches(1);
  k_scale_value<T><<<grid_of(n), kThreads, 0, s>>>(y, x, n, a);
}

template <class T>
void gmres_sub_from(T* y, const T* b, int64_t n, cudaStream_t s) {
  if (n == 0) return;
  count_launches(1);
  k_sub_from<T><<<grid_of(n), kThreads, 0, s>>>(y, b, n);
}

template void gmres_scale_value<double>(double*, const double*, int64_t, double, cudaStream_t);
template void gmres_scale_value<float>(float*, const float*, int64_t, double, cudaStream_t);
template void gmres_sub_from<double>(double*, const double*, int64_t, cudaStream_t);
template void gmres_sub_from<float>(float*, const float*, int64_t, cudaStream_t);
template void gmres_mdot<double>(const double*, int64_t, int, const double*, double*, double*, bool, cudaStream_t);
template void gmres_mdot<float>(const float*, int64_t, int, const float*, double*, double*, bool, cudaStream_t);
template void gmres_maxpy<double>(double*, const double*, int64_t, int, const double*, double, cudaStream_t);
template void gmres_maxpy<float>(float*, const float*, int64_t, int, const double*, double, cudaStream_t);
template void gmres_scale<double>(double*, const double*, int64_t, const double*, cudaStream_t);
template void gmres_scale<float>(float*, const float*, int64_t, const double*, cudaStream_t);

}  // namespace dcgpu
