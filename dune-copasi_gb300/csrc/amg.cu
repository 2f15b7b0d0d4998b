#include "amg.hpp"

#include <algorithm>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "blockops.cuh"
#include "sellrow.cuh"

namespace dcgpu {

namespace {

constexpr int kT = 256;

inline int blocks_for(int64_t n) {
  int64_t b = (n + kT - 1) / kT;
  return static_cast<int>(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}
// blocks of kT threads for a warp per slice
inline int blocks_for_slices(int64_t nslices) { return blocks_for(nslices * 32); }

__device__ __forceinline__ bool skip(const double* sc, int slot) { return sc && sc[slot] != 0.0; }

// coarse block entry = sum of the listed fine blocks' entries (fixed order)
__global__ void k_galerkin(int64_t n_entries, int bs2, const int32_t* __restrict__ gal_ptr,
                           const int32_t* __restrict__ gal_src, const double* __restrict__ fine,
                           double* __restrict__ coarse) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n_entries; t += stride) {
    const int64_t k = t / bs2;
    const int e = static_cast<int>(t % bs2);
    double acc = 0.0;
    for (int32_t q = gal_ptr[k]; q < gal_ptr[k + 1]; ++q) acc += fine[static_cast<int64_t>(gal_src[q]) * bs2 + e];
    coarse[t] = acc;
  }
}

// L1-Jacobi inverse: (A_ii + diag(sum over j != i of |A_ij| by row))^-1
template <int B>
__global__ void k_l1_setup(int64_t nrows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ diag,
                           const double* __restrict__ val, double* __restrict__ sinv, float* __restrict__ sinv32,
                           int* status) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nrows; i += stride) {
    double a[B][B], inv[B][B];
    load_block<B>(val + static_cast<int64_t>(diag[i]) * B * B, a);
    for (int32_t e = rowptr[i]; e < rowptr[i + 1]; ++e) {
      if (e == diag[i]) continue;
      const double* blk = val + static_cast<int64_t>(e) * B * B;
#pragma unroll
      for (int s = 0; s < B; ++s) {
        double m = 0.0;
#pragma unroll
        for (int q = 0; q < B; ++q) m += fabs(blk[s * B + q]);
        a[s][s] += a[s][s] < 0.0 ? -m : m;
      }
    }
    if (!invert_block<B>(a, inv)) {
      atomicExch(status, 1);
      continue;
    }
    store_block<B>(sinv + i * B * B, inv);
    if (sinv32) {
#pragma unroll
      for (int s = 0; s < B; ++s)
#pragma unroll
        for (int q = 0; q < B; ++q) sinv32[i * B * B + s * B + q] = static_cast<float>(inv[s][q]);
    }
  }
}

// x = omega S r   (S: the smoother's inverse blocks)
template <int B, class T>
__global__ void k_smooth_first(int64_t nrows, const T* __restrict__ sinv, const T* __restrict__ r, T* __restrict__ x,
                               T omega, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nrows; i += stride) {
    const T* d = sinv + i * B * B;
    T rv[B];
#pragma unroll
    for (int q = 0; q < B; ++q) rv[q] = r[i * B + q];
#pragma unroll
    for (int s = 0; s < B; ++s) {
      T acc = T(0);
#pragma unroll
      for (int q = 0; q < B; ++q) acc += d[s * B + q] * rv[q];
      x[i * B + s] = omega * acc;
    }
  }
}

// x_out = x_in + omega S (r - A x_in)   (SELL-32, lane per row)
template <int B, class T>
__global__ void k_smooth_more(Sell S, const T* __restrict__ val, const T* __restrict__ sinv, const T* __restrict__ r,
                              const T* __restrict__ xin, T* __restrict__ xout, T omega, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const SliceLoop L;
  for (int64_t sl = L.first; sl < S.nslices; sl += L.stride) {
    const int64_t i = sl * 32 + L.lane;
    if (i >= S.nrows) continue;
    T acc[B];
#pragma unroll
    for (int s = 0; s < B; ++s) acc[s] = T(0);
    sell_row_apply<B, T>(S, sl, L.lane, val, [](int32_t) { return true; },
                         [&](int32_t c, T (&xv)[B]) {
#pragma unroll
                           for (int q = 0; q < B; ++q) xv[q] = xin[static_cast<int64_t>(c) * B + q];
                         },
                         acc);
    T t[B];
#pragma unroll
    for (int s = 0; s < B; ++s) t[s] = r[i * B + s] - acc[s];
    const T* d = sinv + i * B * B;
#pragma unroll
    for (int s = 0; s < B; ++s) {
      T a = T(0);
#pragma unroll
      for (int q = 0; q < B; ++q) a += d[s * B + q] * t[q];
      xout[i * B + s] = xin[i * B + s] + omega * a;
    }
  }
}

// u = r - A x   (SELL-32, lane per row)
template <int B, class T>
__global__ void k_residual(Sell S, const T* __restrict__ val, const T* __restrict__ x, const T* __restrict__ r,
                           T* __restrict__ u, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const SliceLoop L;
  for (int64_t sl = L.first; sl < S.nslices; sl += L.stride) {
    const int64_t i = sl * 32 + L.lane;
    if (i >= S.nrows) continue;
    T acc[B];
#pragma unroll
    for (int s = 0; s < B; ++s) acc[s] = T(0);
    sell_row_apply<B, T>(S, sl, L.lane, val, [](int32_t) { return true; },
                         [&](int32_t c, T (&xv)[B]) {
#pragma unroll
                           for (int q = 0; q < B; ++q) xv[q] = x[static_cast<int64_t>(c) * B + q];
                         },
                         acc);
#pragma unroll
    for (int s = 0; s < B; ++s) u[i * B + s] = r[i * B + s] - acc[s];
  }
}

// x = y + omega S (r - A y) with y = t + P xc, formed on the fly (coarse correction and
// post-smoothing in one pass over A; SELL-32, lane per row)
template <int B, class T>
__global__ void k_prolong_smooth(Sell S, const T* __restrict__ val, const T* __restrict__ sinv,
                                 const int32_t* __restrict__ agg, const T* __restrict__ xc, const T* __restrict__ t,
                                 const T* __restrict__ r, T* __restrict__ x, T omega, T cs, const double* sc,
                                 int slot) {
  if (skip(sc, slot)) return;
  const SliceLoop L;
  for (int64_t sl = L.first; sl < S.nslices; sl += L.stride) {
    const int64_t i = sl * 32 + L.lane;
    if (i >= S.nrows) continue;
    T acc[B];
#pragma unroll
    for (int s = 0; s < B; ++s) acc[s] = T(0);
    sell_row_apply<B, T>(S, sl, L.lane, val, [](int32_t) { return true; },
                         [&](int32_t c, T (&xv)[B]) {
                           const T* tj = t + static_cast<int64_t>(c) * B;
                           const T* cj = xc + static_cast<int64_t>(agg[c]) * B;
#pragma unroll
                           for (int q = 0; q < B; ++q) xv[q] = tj[q] + cs * cj[q];
                         },
                         acc);
    const T* ci = xc + static_cast<int64_t>(agg[i]) * B;
    T res[B];
#pragma unroll
    for (int s = 0; s < B; ++s) res[s] = r[i * B + s] - acc[s];
    const T* d = sinv + i * B * B;
#pragma unroll
    for (int s = 0; s < B; ++s) {
      T a = T(0);
#pragma unroll
      for (int q = 0; q < B; ++q) a += d[s * B + q] * res[q];
      x[i * B + s] = t[i * B + s] + cs * ci[s] + omega * a;
    }
  }
}

// Warp per row on the BSR values (small levels): lanes take the row's blocks in turn, the
// partial products are summed over the warp (fixed butterfly order), and lane 0 finishes
// the row.  MODE 0: out = r - A x.  MODE 1: out = y + omega S (r - A y) with y = x + cs P xc
// (x: the pre-smoothed iterate).  MODE 2: out = x + omega S (r - A x).
template <int B, class T, int MODE>
__global__ void k_rows_warp(int64_t nrows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                            const T* __restrict__ val, const T* __restrict__ sinv, const int32_t* __restrict__ agg,
                            const T* __restrict__ xc, const T* __restrict__ x, const T* __restrict__ r,
                            T* __restrict__ out, T omega, T cs, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const SliceLoop L;  // here: one row per warp
  for (int64_t i = L.first; i < nrows; i += L.stride) {
    T acc[B];
#pragma unroll
    for (int s = 0; s < B; ++s) acc[s] = T(0);
    for (int32_t e = rowptr[i] + L.lane; e < rowptr[i + 1]; e += 32) {
      const int32_t c = colidx[e];
      T xv[B];
#pragma unroll
      for (int q = 0; q < B; ++q) {
        xv[q] = x[static_cast<int64_t>(c) * B + q];
        if (MODE == 1) xv[q] += cs * xc[static_cast<int64_t>(agg[c]) * B + q];
      }
      const T* blk = val + static_cast<int64_t>(e) * B * B;
#pragma unroll
      for (int s = 0; s < B; ++s)
#pragma unroll
        for (int q = 0; q < B; ++q) acc[s] += blk[s * B + q] * xv[q];
    }
#pragma unroll
    for (int s = 0; s < B; ++s)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[s] += __shfl_xor_sync(0xffffffffu, acc[s], o);
    if (L.lane != 0) continue;
    T res[B];
#pragma unroll
    for (int s = 0; s < B; ++s) res[s] = r[i * B + s] - acc[s];
    if (MODE == 0) {
#pragma unroll
      for (int s = 0; s < B; ++s) out[i * B + s] = res[s];
      continue;
    }
    const T* d = sinv + i * B * B;
#pragma unroll
    for (int s = 0; s < B; ++s) {
      T a = T(0);
#pragma unroll
      for (int q = 0; q < B; ++q) a += d[s * B + q] * res[q];
      T y = x[i * B + s];
      if (MODE == 1) y += cs * xc[static_cast<int64_t>(agg[i]) * B + s];
      out[i * B + s] = y + omega * a;
    }
  }
}

// rc[I] = sum of u over the rows of aggregate I: warp per aggregate, fixed butterfly order
template <int B, class T>
__global__ void k_restrict_warp(int64_t ncoarse, const int32_t* __restrict__ agg_ptr,
                                const int32_t* __restrict__ agg_rows, const T* __restrict__ u, T* __restrict__ rc,
                                const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const SliceLoop L;
  for (int64_t I = L.first; I < ncoarse; I += L.stride) {
    T acc[B];
#pragma unroll
    for (int s = 0; s < B; ++s) acc[s] = T(0);
    for (int32_t q = agg_ptr[I] + L.lane; q < agg_ptr[I + 1]; q += 32) {
      const T* ui = u + static_cast<int64_t>(agg_rows[q]) * B;
#pragma unroll
      for (int s = 0; s < B; ++s) acc[s] += ui[s];
    }
#pragma unroll
    for (int s = 0; s < B; ++s)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[s] += __shfl_xor_sync(0xffffffffu, acc[s], o);
    if (L.lane == 0)
#pragma unroll
      for (int s = 0; s < B; ++s) rc[I * B + s] = acc[s];
  }
}

// x += w
template <class T>
__global__ void k_add(int64_t n, const T* __restrict__ w, T* __restrict__ x, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) x[i] += w[i];
}

// x = t + cs P xc (the coarse correction without post-smoothing)
template <int B, class T>
__global__ void k_prolong_to(int64_t nrows, const int32_t* __restrict__ agg, const T* __restrict__ xc,
                             const T* __restrict__ t, T* __restrict__ x, T cs, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int64_t n = nrows * B;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; row < n; row += stride)
    x[row] = t[row] + cs * xc[static_cast<int64_t>(agg[row / B]) * B + row % B];
}

// x += cs P xc
template <int B, class T>
__global__ void k_prolong(int64_t nrows, const int32_t* __restrict__ agg, const T* __restrict__ xc, T* __restrict__ x,
                          T cs, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int64_t n = nrows * B;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; row < n; row += stride)
    x[row] += cs * xc[static_cast<int64_t>(agg[row / B]) * B + row % B];
}

// ---------------------------------------------------------------- dense coarsest solve
template <int B>
__global__ void k_dense_fill(int64_t nrows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                             const double* __restrict__ val, int n, double* __restrict__ dense) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t I = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; I < nrows; I += stride)
    for (int32_t e = rowptr[I]; e < rowptr[I + 1]; ++e)
      for (int s = 0; s < B; ++s)
        for (int q = 0; q < B; ++q)
          dense[(I * B + s) * n + static_cast<int64_t>(colidx[e]) * B + q] = val[static_cast<int64_t>(e) * B * B + s * B + q];
}

constexpr int kLuThreads = 256;

// LU = P A with partial pivoting (row-major, unit lower triangle implicit), one block, the
// matrix in shared memory; perm[i] = the row of A at position i.  status[0] = 1 on a zero
// or non-finite pivot.
__global__ void __launch_bounds__(kLuThreads) k_dense_lu(int n, const double* A, double* LU,
                                                         int32_t* __restrict__ perm_out, int* status) {
  extern __shared__ double a[];
  __shared__ int32_t perm[Amg::kDenseMax];
  __shared__ int s_piv, s_fail;
  for (int q = threadIdx.x; q < n * n; q += kLuThreads) a[q] = A[q];
  for (int q = threadIdx.x; q < n; q += kLuThreads) perm[q] = q;
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x < 32) {  // pivot: largest |a[i][k]| for i >= k, lowest index on ties
      double best = -1.0;
      int bi = k;
      for (int i = k + threadIdx.x; i < n; i += 32) {
        const double v = fabs(a[i * n + k]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (threadIdx.x == 0) {
        s_piv = bi;
        if (!(best > 0.0) || !isfinite(best)) s_fail = 1;
        const int32_t t = perm[k];
        perm[k] = perm[bi];
        perm[bi] = t;
      }
    }
    __syncthreads();
    if (s_fail) break;
    const int p = s_piv;
    if (p != k)
      for (int j = threadIdx.x; j < n; j += kLuThreads) {
        const double t = a[k * n + j];
        a[k * n + j] = a[p * n + j];
        a[p * n + j] = t;
      }
    __syncthreads();
    const double piv = a[k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += kLuThreads) a[i * n + k] /= piv;
    __syncthreads();
    const int m = n - k - 1;
    for (int q = threadIdx.x; q < m * m; q += kLuThreads) {
      const int i = k + 1 + q / m, j = k + 1 + q % m;
      a[i * n + j] -= a[i * n + k] * a[k * n + j];
    }
    __syncthreads();
  }
  if (s_fail) {
    if (threadIdx.x == 0) atomicExch(status, 1);
    return;
  }
  for (int q = threadIdx.x; q < n * n; q += kLuThreads) LU[q] = a[q];
  for (int q = threadIdx.x; q < n; q += kLuThreads) perm_out[q] = perm[q];
}

// column j (block j) of A^-1 from LU = P A: solve L U y = P e_j; written column-major
// (inv_cm[j * n + i] = (A^-1)_ij), fp64 and fp32
__global__ void __launch_bounds__(Amg::kDenseMax) k_dense_inverse(int n, const double* __restrict__ LU,
                                                                  const int32_t* __restrict__ perm,
                                                                  double* __restrict__ inv_cm,
                                                                  float* __restrict__ inv_cm32) {
  __shared__ double y[Amg::kDenseMax];
  const int j = blockIdx.x, i = threadIdx.x;
  if (i < n) y[i] = perm[i] == j ? 1.0 : 0.0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {  // unit lower triangle
    if (i > k && i < n) y[i] -= LU[i * n + k] * y[k];
    __syncthreads();
  }
  for (int k = n - 1; k >= 0; --k) {
    if (i == k) y[k] /= LU[k * n + k];
    __syncthreads();
    if (i < k) y[i] -= LU[i * n + k] * y[k];
    __syncthreads();
  }
  if (i < n) {
    inv_cm[static_cast<int64_t>(j) * n + i] = y[i];
    inv_cm32[static_cast<int64_t>(j) * n + i] = static_cast<float>(y[i]);
  }
}

// x = A^-1 r with the column-major inverse
template <class T>
__global__ void k_dense_apply(int n, const T* __restrict__ inv_cm, const T* __restrict__ r, T* __restrict__ x,
                              const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T acc = T(0);
  for (int j = 0; j < n; ++j) acc += inv_cm[static_cast<int64_t>(j) * n + i] * r[j];
  x[i] = acc;
}

template <class T>
T* pick(const DeviceBuffer<double>& d, const DeviceBuffer<float>& f) {
  if constexpr (std::is_same<T, float>::value) return f.get();
  else return d.get();
}
template <class T>
const T* pickc(const double* d, const float* f) {
  if constexpr (std::is_same<T, float>::value) return f;
  else return d;
}

}  // namespace

void Amg::build(int64_t nrows, int bs, int64_t nnzb, const int32_t* rowptr, const int32_t* colidx,
                const int32_t* diag, const int32_t* group, cudaStream_t s) {
  if (bs < 1 || bs > 8) throw std::runtime_error("multigrid: block size " + std::to_string(bs) + " unsupported");
  levels_.clear();
  bs_ = bs;
  dense_n_ = 0;
  const int64_t target = coarsen_target > 0 ? coarsen_target : std::max<int64_t>(1, kDenseMax / bs);
  {
    Level L0;
    L0.nrows = nrows;
    L0.nnzb = nnzb;
    L0.rowptr = rowptr;
    L0.colidx = colidx;
    L0.diag = diag;
    L0.group = group;
    levels_.push_back(std::move(L0));
  }
  while (static_cast<int>(levels_.size()) < max_levels && levels_.back().nrows > target) {
    Level& f = levels_.back();
    DeviceGraph g;
    g.n = f.nrows;
    g.rowptr = f.rowptr;
    g.colidx = f.colidx;
    g.group = f.group;
    f.agg.resize(static_cast<size_t>(f.nrows));
    const int64_t na = aggregate_mis(g, mis_distance, f.agg.get(), s);
    if (na >= 0.9 * static_cast<double>(f.nrows)) {  // coarsening stalled: this level is the coarsest
      f.agg.resize(0);
      break;
    }
    Level c;
    coarse_structure(g, f.agg.get(), na, &c.own, s);
    c.nrows = na;
    c.nnzb = c.own.nnzb;
    c.rowptr = c.own.rowptr.get();
    c.colidx = c.own.colidx.get();
    c.diag = c.own.diag.get();
    c.group = c.own.group.get();
    levels_.push_back(std::move(c));
  }
  const int64_t last_n = levels_.back().nrows * bs;
  if (last_n <= kDenseMax) {
    dense_n_ = static_cast<int>(last_n);
    const size_t n2 = static_cast<size_t>(dense_n_) * dense_n_;
    dense_.resize(n2);
    dinvd_.resize(n2);
    dinvf_.resize(n2);
    dense_piv_.resize(static_cast<size_t>(dense_n_));
    // the attribute is the kernel's, shared by every multigrid of the process: set once to
    // the largest dense level, so no instance lowers it under another's launch
    static const bool attr_set = [] {
      cuda_check(cudaFuncSetAttribute(k_dense_lu, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(sizeof(double) * kDenseMax * kDenseMax)),
                 "multigrid dense solve");
      return true;
    }();
    (void)attr_set;
  }
  const size_t b2 = static_cast<size_t>(bs) * bs;
  for (size_t l = 0; l < levels_.size(); ++l) {
    Level& L = levels_[l];
    const size_t nv = static_cast<size_t>(L.nrows) * bs;
    if (l > 0) {
      L.val_o.resize(static_cast<size_t>(L.nnzb) * b2);
      L.dinv_o.resize(static_cast<size_t>(L.nrows) * b2);
      L.val = L.val_o.get();
      L.dinv = L.dinv_o.get();
    }
    L.x.resize(nv);
    L.t.resize(nv);
    L.rc.resize(nv);
    const bool smoothed = !(l + 1 == levels_.size() && dense_n_ > 0);
    L.warp_rows = smoothed && L.nrows < warp_rows_below;
    if (smoothed && !L.warp_rows) sell_structure(L.nrows, L.rowptr, L.colidx, &L.sell, s);
    if (smoothed && smoother == Smoother::L1Jacobi) L.sinv_o.resize(static_cast<size_t>(L.nrows) * b2);
    if (smoothed && (smoother == Smoother::GaussSeidel || smoother == Smoother::Ilu0)) {
      L.gs = std::make_unique<ColorPrecond>();
      L.gs->build(smoother == Smoother::Ilu0 ? ColorPrecond::Kind::Ilu0 : ColorPrecond::Kind::Sor, L.nrows, bs, L.nnzb,
                  L.rowptr, L.colidx, L.diag, s);
      L.gs->omega = smoother == Smoother::Ilu0 ? 1.0 : omega;
      if (smoother == Smoother::Ilu0) L.w.resize(nv);
    }
  }
  cuda_check(cudaStreamSynchronize(s), "multigrid set-up");
}

std::string Amg::describe() const {
  static const char* names[] = {"jacobi", "l1jacobi", "gauss_seidel", "ilu0"};
  std::string o = "{\"type\": \"AMG\", \"smoother\": \"" + std::string(names[static_cast<int>(smoother)]) +
                  "\", \"aggregation_distance\": " + std::to_string(mis_distance) + ", \"levels\": [";
  for (size_t l = 0; l < levels_.size(); ++l) {
    const Level& L = levels_[l];
    const bool dense = l + 1 == levels_.size() && dense_n_ > 0;
    o += (l ? ", " : "") + std::string("{\"rows\": ") + std::to_string(L.nrows) + ", \"blocks\": " +
         std::to_string(L.nnzb) + ", \"kernels\": \"" + (dense ? "dense" : L.warp_rows ? "warp_per_row" : "sell32") +
         "\"}";
  }
  return o + "]}";
}

std::vector<double> Amg::values_host(int l) const {
  const Level& L = levels_[l];
  std::vector<double> h(static_cast<size_t>(L.nnzb) * bs_ * bs_);
  if (!h.empty())
    cuda_check(cudaMemcpy(h.data(), L.val, h.size() * sizeof(double), cudaMemcpyDeviceToHost), "multigrid values");
  return h;
}
std::vector<int32_t> Amg::rowptr_host(int l) const {
  const Level& L = levels_[l];
  std::vector<int32_t> h(static_cast<size_t>(L.nrows) + 1);
  cuda_check(cudaMemcpy(h.data(), L.rowptr, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost), "multigrid pattern");
  return h;
}
std::vector<int32_t> Amg::colidx_host(int l) const {
  const Level& L = levels_[l];
  std::vector<int32_t> h(static_cast<size_t>(L.nnzb));
  if (!h.empty())
    cuda_check(cudaMemcpy(h.data(), L.colidx, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost), "multigrid pattern");
  return h;
}

void Amg::setup(const double* fine_vals, const double* fine_dinv, const float* fine_dinv32, bool fp32, int* status,
                cudaStream_t s, const Sell* fine_sell, const float* fine_sell32) {
  if (levels_.empty()) return;
  levels_[0].val = fine_vals;
  levels_[0].dinv = fine_dinv;
  levels_[0].dinv32 = fine_dinv32;
  const int bs2 = bs_ * bs_;
  for (size_t l = 1; l < levels_.size(); ++l) {
    Level& f = levels_[l - 1];
    Level& c = levels_[l];
    const int64_t ne = c.nnzb * bs2;
    count_launches(1);
    k_galerkin<<<blocks_for(ne), kT, 0, s>>>(ne, bs2, c.own.gal_ptr.get(), c.own.gal_src.get(), f.val, c.val_o.get());
    Bsr A;
    A.nrows = static_cast<int>(c.nrows);
    A.bs = bs_;
    A.nnzb = c.nnzb;
    A.rowptr = c.rowptr;
    A.colidx = c.colidx;
    A.val = c.val_o.get();
    if (fp32 && c.dinv32_o.size() != c.dinv_o.size()) c.dinv32_o.resize(c.dinv_o.size());
    block_jacobi_setup(A, c.diag, c.dinv_o.get(), status, s, fp32 ? c.dinv32_o.get() : nullptr);
    c.dinv32 = fp32 ? c.dinv32_o.get() : nullptr;
  }
  // SELL-32 copies of the values in the precision the cycle runs in (level 0 may borrow the
  // caller's)
  {
    Level& L0 = levels_[0];
    L0.ext = fp32 && fine_sell && fine_sell32 && !L0.warp_rows && L0.sell.nslices > 0 &&
             fine_sell->nrows == L0.nrows && fine_sell->bs == bs_;
    if (L0.ext) {
      L0.ext_view = *fine_sell;
      L0.ext_sv32 = fine_sell32;
      L0.sv32.resize(0);
    }
  }
  for (auto& L : levels_) {
    if (L.warp_rows && fp32) {
      const size_t nb = static_cast<size_t>(L.nnzb) * bs2;
      if (L.val32_o.size() != nb) L.val32_o.resize(nb);
      to_float(static_cast<int64_t>(nb), L.val, L.val32_o.get(), s);
    }
    if (L.sell.nslices == 0 || L.ext) continue;
    const size_t nv = static_cast<size_t>(L.sell.nslots) * 32 * bs2;
    if (fp32) {
      if (L.sv32.size() != nv) L.sv32.resize(nv);
      sell_values(L.sell, bs_, L.val, L.sv32.get(), s);
    } else {
      if (L.sv64.size() != nv) L.sv64.resize(nv);
      sell_values(L.sell, bs_, L.val, L.sv64.get(), s);
    }
  }
  if (fp32)
    for (auto& L : levels_)
      if (L.x32.size() != L.x.size()) {
        L.x32.resize(L.x.size());
        L.t32.resize(L.t.size());
        L.rc32.resize(L.rc.size());
        L.w32.resize(L.w.size());
      }
  fp32_ = fp32;
  // smoothers
  for (size_t l = 0; l < levels_.size(); ++l) {
    Level& L = levels_[l];
    if (L.sinv_o.size()) {
      if (fp32 && L.sinv32_o.size() != L.sinv_o.size()) L.sinv32_o.resize(L.sinv_o.size());
      count_launches(1);
#define DC_L1(B)                                                                                             \
  case B:                                                                                                    \
    k_l1_setup<B><<<blocks_for(L.nrows), kT, 0, s>>>(L.nrows, L.rowptr, L.diag, L.val, L.sinv_o.get(),      \
                                                     fp32 ? L.sinv32_o.get() : nullptr, status);             \
    break;
      switch (bs_) { DC_L1(1) DC_L1(2) DC_L1(3) DC_L1(4) DC_L1(5) DC_L1(6) DC_L1(7) DC_L1(8) }
#undef DC_L1
    }
    if (L.gs) L.gs->setup(L.val, L.dinv, L.dinv32, fp32, status, s, L.ext ? &L.ext_view : nullptr, L.ext_sv32);
  }
  // dense coarsest solve
  if (dense_n_ > 0) {
    const Level& c = levels_.back();
    const int n = dense_n_;
    cuda_check(cudaMemsetAsync(dense_.get(), 0, static_cast<size_t>(n) * n * sizeof(double), s), "multigrid");
    count_launches(3);
#define DC_DF(B) \
  case B: k_dense_fill<B><<<blocks_for(c.nrows), kT, 0, s>>>(c.nrows, c.rowptr, c.colidx, c.val, n, dense_.get()); break;
    switch (bs_) { DC_DF(1) DC_DF(2) DC_DF(3) DC_DF(4) DC_DF(5) DC_DF(6) DC_DF(7) DC_DF(8) }
#undef DC_DF
    // factor in place: the LU overwrites the assembled matrix
    k_dense_lu<<<1, kLuThreads, static_cast<size_t>(n) * n * sizeof(double), s>>>(n, dense_.get(), dense_.get(),
                                                                                 dense_piv_.get(), status);
    k_dense_inverse<<<n, kDenseMax, 0, s>>>(n, dense_.get(), dense_piv_.get(), dinvd_.get(), dinvf_.get());
  }
}

template <class T>
void Amg::cycle(int l, const T* r, T* x, const double* sc, int slot, cudaStream_t s) const {
  const Level& a = levels_[l];
  const int64_t n = a.nrows;
  const T* A = a.warp_rows ? pickc<T>(a.val, a.val32_o.get())
                           : a.ext ? pickc<T>(nullptr, a.ext_sv32) : pick<T>(a.sv64, a.sv32);
  const T* D = pickc<T>(a.dinv, a.dinv32);
  const Sell SA = a.ext ? a.ext_view : a.sell.view(bs_);
  const int gw = blocks_for(n * 32);  // warp per row
  const T w = static_cast<T>(omega);
  const T cs = static_cast<T>(correction);
  T* t = pick<T>(a.t, a.t32);
  const bool last = l + 1 == static_cast<int>(levels_.size());
#define DC_BS(KERNEL_CALL)                                                                                    \
  switch (bs_) {                                                                                              \
    case 1: { constexpr int B = 1; KERNEL_CALL; } break;                                                      \
    case 2: { constexpr int B = 2; KERNEL_CALL; } break;                                                      \
    case 3: { constexpr int B = 3; KERNEL_CALL; } break;                                                      \
    case 4: { constexpr int B = 4; KERNEL_CALL; } break;                                                      \
    case 5: { constexpr int B = 5; KERNEL_CALL; } break;                                                      \
    case 6: { constexpr int B = 6; KERNEL_CALL; } break;                                                      \
    case 7: { constexpr int B = 7; KERNEL_CALL; } break;                                                      \
    default: { constexpr int B = 8; KERNEL_CALL; } break;                                                     \
  }
  // u = r - A v
  auto residual = [&](const T* v, T* u) {
    if (a.warp_rows)
      DC_BS((k_rows_warp<B, T, 0><<<gw, kT, 0, s>>>(n, a.rowptr, a.colidx, A, nullptr, nullptr, nullptr, v, r, u, w,
                                                     cs, sc, slot)))
    else
      DC_BS((k_residual<B, T><<<blocks_for_slices(SA.nslices), kT, 0, s>>>(SA, A, v, r, u, sc, slot)))
  };
  if (last) {
    if (dense_n_ > 0) {
      count_launches(1);
      k_dense_apply<T><<<(dense_n_ + 31) / 32, 32, 0, s>>>(dense_n_, pick<T>(dinvd_, dinvf_), r, x, sc, slot);
      return;
    }
    // coarsening stalled above the dense limit: damped block-Jacobi sweeps
    count_launches(1);
    DC_BS((k_smooth_first<B, T><<<blocks_for(n), kT, 0, s>>>(n, D, r, x, w, sc, slot)));
    for (int k = 1; k < coarse_sweeps; ++k) {
      count_launches(2);
      if (a.warp_rows)
        DC_BS((k_rows_warp<B, T, 2><<<gw, kT, 0, s>>>(n, a.rowptr, a.colidx, A, D, nullptr, nullptr, x, r, t, w, cs,
                                                       sc, slot)))
      else
        DC_BS((k_smooth_more<B, T><<<blocks_for_slices(SA.nslices), kT, 0, s>>>(SA, A, D, r, x, t, w, sc, slot)))
      cuda_check(cudaMemcpyAsync(x, t, static_cast<size_t>(n) * bs_ * sizeof(T), cudaMemcpyDeviceToDevice, s),
                 "multigrid");
    }
    return;
  }
  const Level& c = levels_[l + 1];
  T* u = t;  // residual scratch (Gauss-Seidel) / smoothed iterate (Jacobi)
  T* xc = pick<T>(c.x, c.x32);
  T* rc = pick<T>(c.rc, c.rc32);
  if (smoother == Smoother::Ilu0) {
    T* w = pick<T>(a.w, a.w32);
    a.gs->apply(r, x, sc, slot, s);
    count_launches(2);
    residual(x, u);
    DC_BS((k_restrict_warp<B, T><<<blocks_for(c.nrows * 32), kT, 0, s>>>(c.nrows, c.own.agg_ptr.get(),
                                                                         c.own.agg_rows.get(), u, rc, sc, slot)));
    cycle<T>(l + 1, rc, xc, sc, slot, s);
    count_launches(3);
    DC_BS((k_prolong<B, T><<<blocks_for(n * bs_), kT, 0, s>>>(n, a.agg.get(), xc, x, cs, sc, slot)));
    residual(x, u);
    a.gs->apply(u, w, sc, slot, s);
    k_add<T><<<blocks_for(n * bs_), kT, 0, s>>>(n * bs_, w, x, sc, slot);
    return;
  }
  if (smoother == Smoother::GaussSeidel) {
    a.gs->template sor_sweep<T>(r, x, true, true, sc, slot, s);
    count_launches(2);
    residual(x, u);
    DC_BS((k_restrict_warp<B, T><<<blocks_for(c.nrows * 32), kT, 0, s>>>(c.nrows, c.own.agg_ptr.get(),
                                                                         c.own.agg_rows.get(), u, rc, sc, slot)));
    cycle<T>(l + 1, rc, xc, sc, slot, s);
    count_launches(1);
    DC_BS((k_prolong<B, T><<<blocks_for(n * bs_), kT, 0, s>>>(n, a.agg.get(), xc, x, cs, sc, slot)));
    a.gs->template sor_sweep<T>(r, x, false, false, sc, slot, s);
    return;
  }
  // (L1-)Jacobi: t = omega S r; u = r - A t (into x as scratch); coarse correction; x = y +
  // omega S (r - A y) with y = t + P xc
  const T* S = smoother == Smoother::L1Jacobi ? pick<T>(a.sinv_o, a.sinv32_o) : D;
  count_launches(3);
  DC_BS((k_smooth_first<B, T><<<blocks_for(n), kT, 0, s>>>(n, S, r, t, w, sc, slot)));
  residual(t, x);
  DC_BS((k_restrict_warp<B, T><<<blocks_for(c.nrows * 32), kT, 0, s>>>(c.nrows, c.own.agg_ptr.get(),
                                                                       c.own.agg_rows.get(), x, rc, sc, slot)));
  cycle<T>(l + 1, rc, xc, sc, slot, s);
  if (l < w_levels) {
    // a second coarse-grid correction (W-cycle on this level): t += cs P xc, then the
    // restricted residual of t and another coarse solve
    count_launches(2);
    DC_BS((k_prolong<B, T><<<blocks_for(n * bs_), kT, 0, s>>>(n, a.agg.get(), xc, t, cs, sc, slot)));
    residual(t, x);
    DC_BS((k_restrict_warp<B, T><<<blocks_for(c.nrows * 32), kT, 0, s>>>(c.nrows, c.own.agg_ptr.get(),
                                                                         c.own.agg_rows.get(), x, rc, sc, slot)));
    cycle<T>(l + 1, rc, xc, sc, slot, s);
  }
  count_launches(1);
  if (l == 0 && !finest_post_smoothing)
    DC_BS((k_prolong_to<B, T><<<blocks_for(n * bs_), kT, 0, s>>>(n, a.agg.get(), xc, t, x, cs, sc, slot)))
  else if (a.warp_rows)
    DC_BS((k_rows_warp<B, T, 1><<<gw, kT, 0, s>>>(n, a.rowptr, a.colidx, A, S, a.agg.get(), xc, t, r, x, w, cs, sc,
                                                   slot)))
  else
    DC_BS((k_prolong_smooth<B, T><<<blocks_for_slices(SA.nslices), kT, 0, s>>>(SA, A, S, a.agg.get(), xc, t, r, x, w,
                                                                                cs, sc, slot)))
#undef DC_BS
}

template <class T>
void Amg::apply_t(const T* r, T* z, const double* sc, int done_slot, cudaStream_t s) const {
  if (levels_.empty()) throw std::runtime_error("multigrid: not built");
  if ((std::is_same<T, float>::value) != fp32_)
    throw std::runtime_error("multigrid: applied in another precision than it was set up for");
  cycle<T>(0, r, z, sc, done_slot, s);
}

void Amg::apply(const double* r, double* z, const double* sc, int done_slot, cudaStream_t s) const {
  apply_t<double>(r, z, sc, done_slot, s);
}
void Amg::apply(const float* r, float* z, const double* sc, int done_slot, cudaStream_t s) const {
  apply_t<float>(r, z, sc, done_slot, s);
}

}  // namespace dcgpu
