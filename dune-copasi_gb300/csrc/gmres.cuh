// Vector kernels of the restarted GMRES solver (see gmres.cu; the iteration itself is
// driven by Solver::gmres_run).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace dcgpu {

constexpr int kGmresBlocks = 608;

// out[i] = V_i . w for i < k (accumulate: out[i] += ...); partial holds kGmresBlocks * k doubles
template <class T>
void gmres_mdot(const T* V, int64_t n, int k, const T* w, double* out, double* partial, bool accumulate,
                cudaStream_t s);
// w += sign * sum_{i<k} h[i] V_i  (h on the device)
template <class T>
void gmres_maxpy(T* w, const T* V, int64_t n, int k, const double* h, double sign, cudaStream_t s);
// y = x / by[0]  (by on the device)
template <class T>
void gmres_scale(T* y, const T* x, int64_t n, const double* by, cudaStream_t s);
// y = a x  (a from the host)
template <class T>
void gmres_scale_value(T* y, const T* x, int64_t n, double a, cudaStream_t s);
// y = b - y
template <class T>
void gmres_sub_from(T* y, const T* b, int64_t n, cudaStream_t s);

}  // namespace dcgpu
