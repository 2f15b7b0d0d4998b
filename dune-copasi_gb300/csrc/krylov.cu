#include "krylov.cuh"

#include "precond.hpp"

#include <stdexcept>
#include <string>

namespace dcgpu {

namespace {

constexpr int kThreads = kReduceThreads;
constexpr int kWarps = kThreads / 32;

template <int NSUM>
__device__ __forceinline__ void block_sum_to_thread0(double (&acc)[NSUM], double (*sh)[kWarps]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NSUM; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NSUM; ++k) {
      double v = 0.0;
      for (int w = 0; w < kWarps; ++w) v += sh[k][w];
      acc[k] = v;
    }
  }
  __syncthreads();
}

// Deterministic grid reduction: partial sums per block, the last block to finish adds them
// in index order.  Returns true in the last block, where thread 0 holds the totals in acc.
template <int NSUM>
__device__ __forceinline__ bool grid_sum(double (&acc)[NSUM], ReduceScratch rs) {
  __shared__ double sh[NSUM][kWarps];
  __shared__ bool last;
  block_sum_to_thread0<NSUM>(acc, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NSUM; ++k) rs.partial[blockIdx.x * 4 + k] = acc[k];
    __threadfence();
    const unsigned prev = atomicAdd(rs.counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NSUM; ++k) acc[k] = 0.0;
  for (int b = threadIdx.x; b < static_cast<int>(gridDim.x); b += blockDim.x)
#pragma unroll
    for (int k = 0; k < NSUM; ++k) acc[k] += __ldcg(&rs.partial[b * 4 + k]);
  block_sum_to_thread0<NSUM>(acc, sh);
  if (threadIdx.x == 0) *rs.counter = 0u;
  return threadIdx.x == 0;
}

// The same from the threads' partial sums in the vector precision A: a thread accumulates
// its few elements in A (GB300's FP64 rate is 1/58 of its FP32 rate; a per-element FP64
// product and conversion made the fp32 solve's dot products FP64-bound), the sums across
// threads and blocks are FP64.  The totals are left in tot (thread 0 of the last block).
template <int NSUM, class A>
__device__ __forceinline__ bool grid_sum(const A (&part)[NSUM], double (&tot)[NSUM], ReduceScratch rs) {
  __shared__ double sh[NSUM][kWarps];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // warp sums in A, one conversion per warp
#pragma unroll
  for (int k = 0; k < NSUM; ++k) {
    A v = part[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][warp] = static_cast<double>(v);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NSUM; ++k) {
      double v = 0.0;
      for (int w = 0; w < kWarps; ++w) v += sh[k][w];
      rs.partial[blockIdx.x * 4 + k] = v;
    }
    __threadfence();
    const unsigned prev = atomicAdd(rs.counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // the last block: warp 0 adds the block partials in index order
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NSUM; ++k) tot[k] = 0.0;
    for (int b = lane; b < static_cast<int>(gridDim.x); b += 32)
#pragma unroll
      for (int k = 0; k < NSUM; ++k) tot[k] += __ldcg(&rs.partial[b * 4 + k]);
#pragma unroll
    for (int k = 0; k < NSUM; ++k)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tot[k] += __shfl_down_sync(0xffffffffu, tot[k], o);
  }
  if (threadIdx.x == 0) *rs.counter = 0u;
  return threadIdx.x == 0;
}

__device__ __forceinline__ bool done(const double* sc) { return sc[KS_DONE] != 0.0; }

template <class T>
__global__ void __launch_bounds__(kThreads) k_init(T* x, T* r, T* rhat, T* p, T* v, int64_t n, double rel,
                                                   ReduceScratch rs, double* sc) {
  T part[1] = {T(0)};
  double acc[1];
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T ri = r[i];
    rhat[i] = ri;
    p[i] = T(0);
    v[i] = T(0);
    x[i] = T(0);
    part[0] += ri * ri;
  }
  if (grid_sum<1>(part, acc, rs)) {
    const double rr = acc[0];
    sc[KS_RR] = rr;
    sc[KS_RR0] = rr;
    sc[KS_RHO] = rr;
    sc[KS_RHONEW] = rr;
    sc[KS_ALPHA] = 1.0;
    sc[KS_OMEGA] = 1.0;
    sc[KS_BETA] = 1.0;
    sc[KS_TARGET] = rel * rel * rr;
    sc[KS_ITER] = 0.0;
    sc[KS_DONE] = !isfinite(rr) ? kDoneNonFinite : (rr == 0.0 ? kDoneConverged : 0.0);
  }
}

// (1) p = r + beta (p - omega v);  phat = D^-1 p   (one thread per block row; with BJ
// false the preconditioner is applied by a separate multigrid cycle)
template <int B, class T, class V, bool BJ>
__global__ void __launch_bounds__(kThreads) k_update_p(int nrows, T* __restrict__ p, const T* __restrict__ r,
                                                       const T* __restrict__ v, const V* __restrict__ dinv,
                                                       T* __restrict__ phat, const double* sc) {
  if (done(sc)) return;
  const V beta = static_cast<V>(sc[KS_BETA]), omega = static_cast<V>(sc[KS_OMEGA]);
  const int stride = gridDim.x * blockDim.x;
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < nrows; nd += stride) {
    const int64_t o = static_cast<int64_t>(nd) * B;
    V pv[B];
#pragma unroll
    for (int i = 0; i < B; ++i) {
      pv[i] = static_cast<V>(r[o + i]) + beta * (static_cast<V>(p[o + i]) - omega * static_cast<V>(v[o + i]));
      p[o + i] = static_cast<T>(pv[i]);
    }
    if (!BJ) continue;
    const V* d = dinv + static_cast<int64_t>(nd) * B * B;
#pragma unroll
    for (int i = 0; i < B; ++i) {
      V acc = V(0);
#pragma unroll
      for (int j = 0; j < B; ++j) acc += d[i * B + j] * pv[j];
      phat[o + i] = static_cast<T>(acc);
    }
  }
}

// y = A x for one scalar row (block row br, row i inside the block)
template <int B, class T, class V>
__device__ __forceinline__ V row_product(int br, int i, const int32_t* __restrict__ rowptr,
                                         const int32_t* __restrict__ colidx, const V* __restrict__ val,
                                         const T* __restrict__ x) {
  V acc = V(0);
  const int k0 = rowptr[br], k1 = rowptr[br + 1];
  for (int k = k0; k < k1; ++k) {
    const int c = colidx[k];
    const V* blk = val + static_cast<int64_t>(k) * B * B + i * B;
    const T* xc = x + static_cast<int64_t>(c) * B;
#pragma unroll
    for (int j = 0; j < B; ++j) acc += blk[j] * static_cast<V>(xc[j]);
  }
  return acc;
}

// (2) v = A phat;  <rhat, v>;  alpha = rho / <rhat, v>
template <int B, class T, class V>
__global__ void __launch_bounds__(kThreads) k_spmv_rv(int nrows, const int32_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ colidx, const V* __restrict__ val,
                                                      const T* __restrict__ phat, T* __restrict__ v,
                                                      const T* __restrict__ rhat, ReduceScratch rs, double* sc) {
  if (done(sc)) return;
  T part[1] = {T(0)};
  double acc[1];
  const int64_t n = static_cast<int64_t>(nrows) * B;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; row < n; row += stride) {
    const V y = row_product<B, T, V>(static_cast<int>(row / B), static_cast<int>(row % B), rowptr, colidx, val, phat);
    const T yt = static_cast<T>(y);
    v[row] = yt;
    part[0] += rhat[row] * yt;
  }
  if (grid_sum<1>(part, acc, rs)) {
    const double rv = acc[0];
    sc[KS_RV] = rv;
    const double a = sc[KS_RHO] / rv;
    if (!isfinite(rv)) sc[KS_DONE] = kDoneNonFinite;
    else if (rv == 0.0 || !isfinite(a)) sc[KS_DONE] = kDoneBreakdown;
    sc[KS_ALPHA] = isfinite(a) ? a : 0.0;
  }
}

// (2) on the SELL-32 layout: a warp per slice of 32 block rows, a lane per block row
template <int B, class T, class V>
__global__ void __launch_bounds__(kThreads) k_sell_rv(Sell S, const V* __restrict__ val, const T* __restrict__ phat,
                                                      T* __restrict__ v, const T* __restrict__ rhat,
                                                      ReduceScratch rs, double* sc) {
  if (done(sc)) return;
  T part[1] = {T(0)};
  double acc[1];
  const int lane = threadIdx.x & 31;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t sl = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; sl < S.nslices; sl += nw) {
    V y[B];
    sell_lane_rows<B, T, V>(S, sl, lane, val, phat, y);
    const int64_t br = sl * 32 + lane;
    if (br < S.nrows) {
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const T yt = static_cast<T>(y[i]);
        v[br * B + i] = yt;
        part[0] += rhat[br * B + i] * yt;
      }
    }
  }
  if (grid_sum<1>(part, acc, rs)) {
    const double rv = acc[0];
    sc[KS_RV] = rv;
    const double a = sc[KS_RHO] / rv;
    if (!isfinite(rv)) sc[KS_DONE] = kDoneNonFinite;
    else if (rv == 0.0 || !isfinite(a)) sc[KS_DONE] = kDoneBreakdown;
    sc[KS_ALPHA] = isfinite(a) ? a : 0.0;
  }
}

// (3) s = r - alpha v;  shat = D^-1 s (when BJ);  ||s||^2
template <int B, class T, class V, bool BJ>
__global__ void __launch_bounds__(kThreads) k_update_s(int nrows, T* __restrict__ s, const T* __restrict__ r,
                                                       const T* __restrict__ v, const V* __restrict__ dinv,
                                                       T* __restrict__ shat, ReduceScratch rs, double* sc) {
  if (done(sc)) return;
  const V alpha = static_cast<V>(sc[KS_ALPHA]);
  T part[1] = {T(0)};
  double acc[1];
  const int stride = gridDim.x * blockDim.x;
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < nrows; nd += stride) {
    const int64_t o = static_cast<int64_t>(nd) * B;
    V sv[B];
#pragma unroll
    for (int i = 0; i < B; ++i) {
      sv[i] = static_cast<V>(r[o + i]) - alpha * static_cast<V>(v[o + i]);
      const T st = static_cast<T>(sv[i]);
      s[o + i] = st;
      part[0] += st * st;
    }
    if (!BJ) continue;
    const V* d = dinv + static_cast<int64_t>(nd) * B * B;
#pragma unroll
    for (int i = 0; i < B; ++i) {
      V a2 = V(0);
#pragma unroll
      for (int j = 0; j < B; ++j) a2 += d[i * B + j] * sv[j];
      shat[o + i] = static_cast<T>(a2);
    }
  }
  if (grid_sum<1>(part, acc, rs)) sc[KS_SS] = acc[0];
}

// (4) t = A shat;  <t, s>, <t, t>;  omega = <t,s>/<t,t>
template <int B, class T, class V>
__global__ void __launch_bounds__(kThreads) k_spmv_omega(int nrows, const int32_t* __restrict__ rowptr,
                                                         const int32_t* __restrict__ colidx,
                                                         const V* __restrict__ val, const T* __restrict__ shat,
                                                         T* __restrict__ t, const T* __restrict__ s,
                                                         ReduceScratch rs, double* sc) {
  if (done(sc)) return;
  T part[2] = {T(0), T(0)};
  double acc[2];
  const int64_t n = static_cast<int64_t>(nrows) * B;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; row < n; row += stride) {
    const V y = row_product<B, T, V>(static_cast<int>(row / B), static_cast<int>(row % B), rowptr, colidx, val, shat);
    const T yt = static_cast<T>(y);
    t[row] = yt;
    part[0] += yt * s[row];
    part[1] += yt * yt;
  }
  if (grid_sum<2>(part, acc, rs)) {
    sc[KS_TS] = acc[0];
    sc[KS_TT] = acc[1];
    double w = acc[1] != 0.0 ? acc[0] / acc[1] : 0.0;
    if (!isfinite(w)) {
      sc[KS_DONE] = kDoneNonFinite;
      w = 0.0;
    }
    sc[KS_OMEGA] = w;
  }
}

// (4) on the SELL-32 layout
template <int B, class T, class V>
__global__ void __launch_bounds__(kThreads) k_sell_omega(Sell S, const V* __restrict__ val,
                                                         const T* __restrict__ shat, T* __restrict__ t,
                                                         const T* __restrict__ s, ReduceScratch rs, double* sc) {
  if (done(sc)) return;
  T part[2] = {T(0), T(0)};
  double acc[2];
  const int lane = threadIdx.x & 31;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t sl = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; sl < S.nslices; sl += nw) {
    V y[B];
    sell_lane_rows<B, T, V>(S, sl, lane, val, shat, y);
    const int64_t br = sl * 32 + lane;
    if (br < S.nrows) {
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const T yt = static_cast<T>(y[i]);
        t[br * B + i] = yt;
        part[0] += yt * s[br * B + i];
        part[1] += yt * yt;
      }
    }
  }
  if (grid_sum<2>(part, acc, rs)) {
    sc[KS_TS] = acc[0];
    sc[KS_TT] = acc[1];
    double w = acc[1] != 0.0 ? acc[0] / acc[1] : 0.0;
    if (!isfinite(w)) {
      sc[KS_DONE] = kDoneNonFinite;
      w = 0.0;
    }
    sc[KS_OMEGA] = w;
  }
}

// (5) x += alpha phat + omega shat;  r = s - omega t;  ||r||^2, <rhat, r>;  convergence
template <class T>
__global__ void __launch_bounds__(kThreads) k_update_xr(int64_t n, T* __restrict__ x, T* __restrict__ r,
                                                        const T* __restrict__ phat, const T* __restrict__ shat,
                                                        const T* __restrict__ s, const T* __restrict__ t,
                                                        const T* __restrict__ rhat, ReduceScratch rs, double* sc) {
  if (done(sc)) return;
  using C = T;
  const C alpha = static_cast<C>(sc[KS_ALPHA]), omega = static_cast<C>(sc[KS_OMEGA]);
  T part[2] = {T(0), T(0)};
  double acc[2];
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] = x[i] + alpha * phat[i] + omega * shat[i];
    const T ri = s[i] - omega * t[i];
    r[i] = ri;
    part[0] += ri * ri;
    part[1] += rhat[i] * ri;
  }
  if (grid_sum<2>(part, acc, rs)) {
    const double rr = acc[0], rho_new = acc[1];
    sc[KS_RR] = rr;
    sc[KS_RHONEW] = rho_new;
    sc[KS_ITER] += 1.0;
    if (!isfinite(rr) || !isfinite(rho_new)) {
      sc[KS_DONE] = kDoneNonFinite;
      return;
    }
    if (rr <= sc[KS_TARGET]) {
      sc[KS_DONE] = kDoneConverged;
      return;
    }
    const double beta = (rho_new / sc[KS_RHO]) * (sc[KS_ALPHA] / sc[KS_OMEGA]);
    if (rho_new == 0.0 || sc[KS_OMEGA] == 0.0 || !isfinite(beta)) {
      sc[KS_DONE] = kDoneBreakdown;
      return;
    }
    sc[KS_BETA] = beta;
    sc[KS_RHO] = rho_new;
  }
}

inline int grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b > kReduceBlocks) b = kReduceBlocks;
  return static_cast<int>(b < 1 ? 1 : b);
}

// ---------------------------------------------------------------- preconditioned CG
// Slots: KS_RHO = <r, z>, KS_ALPHA, KS_BETA, KS_RR = ||r||^2, KS_TARGET, KS_DONE, KS_ITER.
// Vectors: x, r, p, z (= s), q (= v).

// x = 0, p = 0, ||r||^2, target; with BJ also z = D^-1 r, rho = <r, z>, beta = 0
template <int B, class T, class V, bool BJ>
__global__ void __launch_bounds__(kThreads) k_cg_init(int nrows, T* x, const T* r, T* p, T* z,
                                                      const V* __restrict__ dinv, double rel, ReduceScratch rs,
                                                      double* sc) {
  T part[2] = {T(0), T(0)};
  double acc[2];
  const int stride = gridDim.x * blockDim.x;
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < nrows; nd += stride) {
    const int64_t o = static_cast<int64_t>(nd) * B;
    V rv[B];
#pragma unroll
    for (int i = 0; i < B; ++i) {
      x[o + i] = T(0);
      p[o + i] = T(0);
      rv[i] = static_cast<V>(r[o + i]);
      part[0] += r[o + i] * r[o + i];
    }
    if (!BJ) continue;
    const V* d = dinv + static_cast<int64_t>(nd) * B * B;
#pragma unroll
    for (int i = 0; i < B; ++i) {
      V a = V(0);
#pragma unroll
      for (int j = 0; j < B; ++j) a += d[i * B + j] * rv[j];
      const T zt = static_cast<T>(a);
      z[o + i] = zt;
      part[1] += r[o + i] * zt;
    }
  }
  if (grid_sum<2>(part, acc, rs)) {
    const double rr = acc[0];
    sc[KS_RR] = rr;
    sc[KS_RR0] = rr;
    sc[KS_TARGET] = rel * rel * rr;
    sc[KS_ITER] = 0.0;
    sc[KS_BETA] = 0.0;
    sc[KS_RHO] = BJ ? acc[1] : 0.0;
    sc[KS_DONE] = !isfinite(rr) ? kDoneNonFinite : (rr == 0.0 ? kDoneConverged : 0.0);
  }
}

// p = z + beta p
template <class T>
__global__ void __launch_bounds__(kThreads) k_cg_p(int64_t n, T* __restrict__ p, const T* __restrict__ z,
                                                   const double* sc) {
  if (done(sc)) return;
  const T beta = static_cast<T>(sc[KS_BETA]);
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    p[i] = z[i] + beta * p[i];
}

// x += alpha p; r -= alpha q; ||r||^2 and the convergence test; with BJ also z = D^-1 r,
// <r, z>, beta = <r, z> / rho and rho = <r, z>
template <int B, class T, class V, bool BJ>
__global__ void __launch_bounds__(kThreads) k_cg_update(int nrows, T* __restrict__ x, T* __restrict__ r,
                                                        T* __restrict__ z, const T* __restrict__ p,
                                                        const T* __restrict__ q, const V* __restrict__ dinv,
                                                        ReduceScratch rs, double* sc) {
  if (done(sc)) return;
  const T alpha = static_cast<T>(sc[KS_ALPHA]);
  T part[2] = {T(0), T(0)};
  double acc[2];
  const int stride = gridDim.x * blockDim.x;
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < nrows; nd += stride) {
    const int64_t o = static_cast<int64_t>(nd) * B;
    V rv[B];
#pragma unroll
    for (int i = 0; i < B; ++i) {
      x[o + i] = x[o + i] + alpha * p[o + i];
      const T ri = r[o + i] - alpha * q[o + i];
      r[o + i] = ri;
      rv[i] = static_cast<V>(ri);
      part[0] += ri * ri;
    }
    if (!BJ) continue;
    const V* d = dinv + static_cast<int64_t>(nd) * B * B;
#pragma unroll
    for (int i = 0; i < B; ++i) {
      V a = V(0);
#pragma unroll
      for (int j = 0; j < B; ++j) a += d[i * B + j] * rv[j];
      const T zt = static_cast<T>(a);
      z[o + i] = zt;
      part[1] += rv[i] * zt;
    }
  }
  if (grid_sum<2>(part, acc, rs)) {
    const double rr = acc[0];
    sc[KS_RR] = rr;
    sc[KS_ITER] += 1.0;
    if (!isfinite(rr)) {
      sc[KS_DONE] = kDoneNonFinite;
      return;
    }
    if (rr <= sc[KS_TARGET]) {
      sc[KS_DONE] = kDoneConverged;
      return;
    }
    if (BJ) {
      const double rz = acc[1], beta = rz / sc[KS_RHO];
      if (rz == 0.0 || !isfinite(beta)) {
        sc[KS_DONE] = kDoneBreakdown;
        return;
      }
      sc[KS_BETA] = beta;
      sc[KS_RHO] = rz;
    }
  }
}

// with a separate preconditioner: <r, z>, beta (0 on the first call), rho
template <class T>
__global__ void __launch_bounds__(kThreads) k_cg_rz(int64_t n, const T* __restrict__ r, const T* __restrict__ z,
                                                    ReduceScratch rs, double* sc) {
  if (done(sc)) return;
  T part[1] = {T(0)};
  double acc[1];
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    part[0] += r[i] * z[i];
  if (grid_sum<1>(part, acc, rs)) {
    const double rz = acc[0];
    const bool first = sc[KS_ITER] == 0.0;
    const double beta = first ? 0.0 : rz / sc[KS_RHO];
    if (!isfinite(rz) || rz == 0.0 || !isfinite(beta)) {
      sc[KS_DONE] = isfinite(rz) ? kDoneBreakdown : kDoneNonFinite;
      return;
    }
    sc[KS_BETA] = beta;
    sc[KS_RHO] = rz;
  }
}

}  // namespace

template <class T, class V>
void cg_init(const Bsr& A, const V* dinv, const KrylovVectors<T>& k, double rel, ReduceScratch rs, double* sc,
             cudaStream_t s, const Preconditioner* pc) {
  count_launches(pc ? 2 : 1);
#define DC_CGI(B)                                                                                              \
  case B:                                                                                                      \
    if (pc)                                                                                                   \
      k_cg_init<B, T, V, false><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, k.x, k.r, k.p, k.s, dinv, rel, rs, \
                                                                   sc);                                        \
    else                                                                                                       \
      k_cg_init<B, T, V, true><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, k.x, k.r, k.p, k.s, dinv, rel, rs,  \
                                                                  sc);                                         \
    break;
  switch (A.bs) {
    DC_CGI(1) DC_CGI(2) DC_CGI(3) DC_CGI(4) DC_CGI(5) DC_CGI(6) DC_CGI(7) DC_CGI(8)
    default: throw std::runtime_error("cg: block size " + std::to_string(A.bs) + " unsupported");
  }
#undef DC_CGI
  if (pc) {
    pc->apply(k.r, k.s, sc, KS_DONE, s);
    k_cg_rz<T><<<kReduceBlocks, kThreads, 0, s>>>(static_cast<int64_t>(A.nrows) * A.bs, k.r, k.s, rs, sc);
  }
}

template <class T, class V>
void cg_iteration(const Bsr& A, const V* vals, const V* dinv, const KrylovVectors<T>& k, ReduceScratch rs,
                  double* sc, cudaStream_t s, const Preconditioner* pc, const Sell* sell) {
  const int64_t n = static_cast<int64_t>(A.nrows) * A.bs;
  count_launches(pc ? 4 : 3);
  k_cg_p<T><<<grid_for(n), kThreads, 0, s>>>(n, k.p, k.s, sc);
#define DC_CG(B)                                                                                                  \
  case B:                                                                                                         \
    /* q = A p, alpha = rho / <p, q>: the BiCGSTAB SpMV kernel with rhat = p */                                   \
    if (sell)                                                                                                     \
      k_sell_rv<B, T, V><<<kReduceBlocks, kThreads, 0, s>>>(*sell, vals, k.p, k.v, k.p, rs, sc);                  \
    else                                                                                                          \
      k_spmv_rv<B, T, V><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, A.rowptr, A.colidx, vals, k.p, k.v, k.p, rs, \
                                                            sc);                                                  \
    if (pc)                                                                                                      \
      k_cg_update<B, T, V, false><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, k.x, k.r, k.s, k.p, k.v, dinv, rs, \
                                                                     sc);                                         \
    else                                                                                                          \
      k_cg_update<B, T, V, true><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, k.x, k.r, k.s, k.p, k.v, dinv, rs,  \
                                                                    sc);                                          \
    break;
  switch (A.bs) {
    DC_CG(1) DC_CG(2) DC_CG(3) DC_CG(4) DC_CG(5) DC_CG(6) DC_CG(7) DC_CG(8)
    default: throw std::runtime_error("cg: block size " + std::to_string(A.bs) + " unsupported");
  }
#undef DC_CG
  if (pc) {
    pc->apply(k.r, k.s, sc, KS_DONE, s);
    k_cg_rz<T><<<kReduceBlocks, kThreads, 0, s>>>(n, k.r, k.s, rs, sc);
  }
}

template void cg_init<double, double>(const Bsr&, const double*, const KrylovVectors<double>&, double, ReduceScratch,
                                      double*, cudaStream_t, const Preconditioner*);
template void cg_init<float, float>(const Bsr&, const float*, const KrylovVectors<float>&, double, ReduceScratch,
                                    double*, cudaStream_t, const Preconditioner*);
template void cg_iteration<double, double>(const Bsr&, const double*, const double*, const KrylovVectors<double>&,
                                           ReduceScratch, double*, cudaStream_t, const Preconditioner*, const Sell*);
template void cg_iteration<float, float>(const Bsr&, const float*, const float*, const KrylovVectors<float>&,
                                         ReduceScratch, double*, cudaStream_t, const Preconditioner*, const Sell*);

template <class T>
void krylov_init(const KrylovVectors<T>& k, int64_t n, double rel, ReduceScratch rs, double* sc, cudaStream_t s) {
  count_launches(1);
  k_init<T><<<kReduceBlocks, kThreads, 0, s>>>(k.x, k.r, k.rhat, k.p, k.v, n, rel, rs, sc);
}

template <class T, class V>
void krylov_iteration(const Bsr& A, const V* vals, const V* dinv, const KrylovVectors<T>& k, ReduceScratch rs,
                      double* sc, cudaStream_t s, cudaEvent_t* ev, const Preconditioner* pc, const Sell* sell) {
  const int64_t n = static_cast<int64_t>(A.nrows) * A.bs;
  const int gn = grid_for(A.nrows);
  count_launches(5);
  // inside a stream capture an event record becomes a graph node only with the external flag
  auto mark = [&](int i) {
    if (ev && cudaEventRecordWithFlags(ev[i], s, cudaEventRecordExternal) != cudaSuccess)
      throw std::runtime_error("cudaEventRecord failed");
  };
#define DC_KR(B)                                                                                                 \
  case B:                                                                                                        \
    if (pc) {                                                                                                   \
      k_update_p<B, T, V, false><<<gn, kThreads, 0, s>>>(A.nrows, k.p, k.r, k.v, dinv, k.phat, sc);              \
      pc->apply(k.p, k.phat, sc, KS_DONE, s);                                                                \
    } else {                                                                                                     \
      k_update_p<B, T, V, true><<<gn, kThreads, 0, s>>>(A.nrows, k.p, k.r, k.v, dinv, k.phat, sc);               \
    }                                                                                                            \
    mark(0);                                                                                                     \
    if (sell)                                                                                                    \
      k_sell_rv<B, T, V><<<kReduceBlocks, kThreads, 0, s>>>(*sell, vals, k.phat, k.v, k.rhat, rs, sc);           \
    else                                                                                                         \
      k_spmv_rv<B, T, V><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, A.rowptr, A.colidx, vals, k.phat, k.v,      \
                                                            k.rhat, rs, sc);                                     \
    mark(1);                                                                                                     \
    if (pc) {                                                                                                   \
      k_update_s<B, T, V, false><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, k.s, k.r, k.v, dinv, k.shat, rs,    \
                                                                    sc);                                         \
      pc->apply(k.s, k.shat, sc, KS_DONE, s);                                                                \
    } else {                                                                                                     \
      k_update_s<B, T, V, true><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, k.s, k.r, k.v, dinv, k.shat, rs, sc); \
    }                                                                                                            \
    mark(2);                                                                                                     \
    if (sell)                                                                                                    \
      k_sell_omega<B, T, V><<<kReduceBlocks, kThreads, 0, s>>>(*sell, vals, k.shat, k.t, k.s, rs, sc);           \
    else                                                                                                         \
      k_spmv_omega<B, T, V><<<kReduceBlocks, kThreads, 0, s>>>(A.nrows, A.rowptr, A.colidx, vals, k.shat, k.t,   \
                                                               k.s, rs, sc);                                     \
    mark(3);                                                                                                     \
    break;
  switch (A.bs) {
    DC_KR(1) DC_KR(2) DC_KR(3) DC_KR(4) DC_KR(5) DC_KR(6) DC_KR(7) DC_KR(8)
    default: throw std::runtime_error("krylov: block size " + std::to_string(A.bs) + " unsupported");
  }
#undef DC_KR
  k_update_xr<T><<<kReduceBlocks, kThreads, 0, s>>>(n, k.x, k.r, k.phat, k.shat, k.s, k.t, k.rhat, rs, sc);
}

template void krylov_init<double>(const KrylovVectors<double>&, int64_t, double, ReduceScratch, double*, cudaStream_t);
template void krylov_init<float>(const KrylovVectors<float>&, int64_t, double, ReduceScratch, double*, cudaStream_t);
template void krylov_iteration<double, double>(const Bsr&, const double*, const double*, const KrylovVectors<double>&,
                                               ReduceScratch, double*, cudaStream_t, cudaEvent_t*, const Preconditioner*,
                                               const Sell*);
template void krylov_iteration<float, float>(const Bsr&, const float*, const float*, const KrylovVectors<float>&,
                                             ReduceScratch, double*, cudaStream_t, cudaEvent_t*, const Preconditioner*,
                                             const Sell*);

}  // namespace dcgpu
