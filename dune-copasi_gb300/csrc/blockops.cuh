// Small dense block operations (B x B, row-major) shared by the preconditioner set-ups.
#pragma once

#include <cstdint>

namespace dcgpu {

// inv = a^-1 by Gauss-Jordan elimination with partial pivoting; a is destroyed.  Returns
// false on a zero or non-finite pivot.
template <int B>
__device__ __forceinline__ bool invert_block(double (&a)[B][B], double (&inv)[B][B]) {
#pragma unroll
  for (int i = 0; i < B; ++i)
#pragma unroll
    for (int j = 0; j < B; ++j) inv[i][j] = (i == j) ? 1.0 : 0.0;
#pragma unroll
  for (int c = 0; c < B; ++c) {
    int piv = c;
    double best = fabs(a[c][c]);
#pragma unroll
    for (int i = c + 1; i < B; ++i)
      if (fabs(a[i][c]) > best) {
        best = fabs(a[i][c]);
        piv = i;
      }
    if (best == 0.0 || !isfinite(best)) return false;
    if (piv != c) {
#pragma unroll
      for (int j = 0; j < B; ++j) {
        double t = a[c][j];
        a[c][j] = a[piv][j];
        a[piv][j] = t;
        t = inv[c][j];
        inv[c][j] = inv[piv][j];
        inv[piv][j] = t;
      }
    }
    const double d = 1.0 / a[c][c];
#pragma unroll
    for (int j = 0; j < B; ++j) {
      a[c][j] *= d;
      inv[c][j] *= d;
    }
#pragma unroll
    for (int i = 0; i < B; ++i) {
      if (i == c) continue;
      const double f = a[i][c];
#pragma unroll
      for (int j = 0; j < B; ++j) {
        a[i][j] -= f * a[c][j];
        inv[i][j] -= f * inv[c][j];
      }
    }
  }
  return true;
}

template <int B>
__device__ __forceinline__ void load_block(const double* p, double (&a)[B][B]) {
#pragma unroll
  for (int i = 0; i < B; ++i)
#pragma unroll
    for (int j = 0; j < B; ++j) a[i][j] = p[i * B + j];
}

template <int B>
__device__ __forceinline__ void store_block(double* p, const double (&a)[B][B]) {
#pragma unroll
  for (int i = 0; i < B; ++i)
#pragma unroll
    for (int j = 0; j < B; ++j) p[i * B + j] = a[i][j];
}

// c = a b
template <int B>
__device__ __forceinline__ void mul_block(const double (&a)[B][B], const double (&b)[B][B], double (&c)[B][B]) {
#pragma unroll
  for (int i = 0; i < B; ++i)
#pragma unroll
    for (int j = 0; j < B; ++j) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < B; ++k) s += a[i][k] * b[k][j];
      c[i][j] = s;
    }
}

// c -= a * (block at p)
template <int B>
__device__ __forceinline__ void sub_mul_block(const double (&a)[B][B], const double* p, double (&c)[B][B]) {
  double b[B][B];
  load_block<B>(p, b);
#pragma unroll
  for (int i = 0; i < B; ++i)
#pragma unroll
    for (int j = 0; j < B; ++j) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < B; ++k) s += a[i][k] * b[k][j];
      c[i][j] -= s;
    }
}

}  // namespace dcgpu
