#include "amg.hpp"

#include <algorithm>
#include <numeric>
#include <stdexcept>
#include <string>

namespace dcgpu {

namespace {

constexpr int kT = 256;

inline int blocks_for(int64_t n) {
  int64_t b = (n + kT - 1) / kT;
  return static_cast<int>(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

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

// x = omega D^-1 r
template <int B, class T, class V>
__global__ void k_bj_scale(int nrows, const V* __restrict__ dinv, const T* __restrict__ r, T* __restrict__ x,
                           V omega, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int stride = gridDim.x * blockDim.x;
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < nrows; nd += stride) {
    const int64_t o = static_cast<int64_t>(nd) * B;
    const V* d = dinv + static_cast<int64_t>(nd) * B * B;
    V rv[B];
#pragma unroll
    for (int j = 0; j < B; ++j) rv[j] = static_cast<V>(r[o + j]);
#pragma unroll
    for (int i = 0; i < B; ++i) {
      V acc = V(0);
#pragma unroll
      for (int j = 0; j < B; ++j) acc += d[i * B + j] * rv[j];
      x[o + i] = static_cast<T>(omega * acc);
    }
  }
}

// x += omega D^-1 t
template <int B, class T, class V>
__global__ void k_bj_axpy(int nrows, const V* __restrict__ dinv, const T* __restrict__ t, T* __restrict__ x,
                          V omega, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int stride = gridDim.x * blockDim.x;
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < nrows; nd += stride) {
    const int64_t o = static_cast<int64_t>(nd) * B;
    const V* d = dinv + static_cast<int64_t>(nd) * B * B;
    V tv[B];
#pragma unroll
    for (int j = 0; j < B; ++j) tv[j] = static_cast<V>(t[o + j]);
#pragma unroll
    for (int i = 0; i < B; ++i) {
      V acc = V(0);
#pragma unroll
      for (int j = 0; j < B; ++j) acc += d[i * B + j] * tv[j];
      x[o + i] = static_cast<T>(static_cast<V>(x[o + i]) + omega * acc);
    }
  }
}

// t = r - A x   (one thread per scalar row)
template <int B, class T, class V>
__global__ void k_residual(int nrows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                           const V* __restrict__ val, const T* __restrict__ x, const T* __restrict__ r,
                           T* __restrict__ t, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int64_t n = static_cast<int64_t>(nrows) * B;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; row < n; row += stride) {
    const int br = static_cast<int>(row / B), i = static_cast<int>(row % B);
    V acc = V(0);
    for (int k = rowptr[br]; k < rowptr[br + 1]; ++k) {
      const V* blk = val + static_cast<int64_t>(k) * B * B + i * B;
      const T* xc = x + static_cast<int64_t>(colidx[k]) * B;
#pragma unroll
      for (int j = 0; j < B; ++j) acc += blk[j] * static_cast<V>(xc[j]);
    }
    t[row] = static_cast<T>(static_cast<V>(r[row]) - acc);
  }
}

// rc[I] = sum of t over the rows of aggregate I
template <int B, class T>
__global__ void k_restrict(int ncoarse, const int32_t* __restrict__ agg_ptr, const int32_t* __restrict__ agg_rows,
                           const T* __restrict__ t, T* __restrict__ rc, const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int stride = gridDim.x * blockDim.x;
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < ncoarse; I += stride) {
    T acc[B];
#pragma unroll
    for (int s = 0; s < B; ++s) acc[s] = T(0);
    for (int q = agg_ptr[I]; q < agg_ptr[I + 1]; ++q) {
      const T* ti = t + static_cast<int64_t>(agg_rows[q]) * B;
#pragma unroll
      for (int s = 0; s < B; ++s) acc[s] += ti[s];
    }
#pragma unroll
    for (int s = 0; s < B; ++s) rc[static_cast<int64_t>(I) * B + s] = acc[s];
  }
}

// x[i] += xc[agg[i]]
template <int B, class T>
__global__ void k_prolong(int nrows, const int32_t* __restrict__ agg, const T* __restrict__ xc, T* __restrict__ x,
                          const double* sc, int slot) {
  if (skip(sc, slot)) return;
  const int64_t n = static_cast<int64_t>(nrows) * B;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; row < n; row += stride) {
    const int64_t i = row / B;
    const int s = static_cast<int>(row % B);
    x[row] += xc[static_cast<int64_t>(agg[i]) * B + s];
  }
}

template <int B, class T, class V>
struct Cycle {
  struct L {
    int64_t nrows;
    const int32_t *rowptr, *colidx, *agg, *agg_ptr, *agg_rows;
    const V *val, *dinv;
    T *x, *t, *rc;
    int64_t ncoarse;
  };
  static void run(const std::vector<L>& lv, int l, const T* r, T* x, V omega, int sweeps, const double* sc,
                  int slot, cudaStream_t s) {
    const L& a = lv[l];
    const int n = static_cast<int>(a.nrows);
    const int gb = blocks_for(a.nrows), gr = blocks_for(a.nrows * B);
    count_launches(1);
    k_bj_scale<B, T, V><<<gb, kT, 0, s>>>(n, a.dinv, r, x, omega, sc, slot);
    if (l + 1 == static_cast<int>(lv.size())) {
      for (int k = 1; k < sweeps; ++k) {
        count_launches(2);
        k_residual<B, T, V><<<gr, kT, 0, s>>>(n, a.rowptr, a.colidx, a.val, x, r, a.t, sc, slot);
        k_bj_axpy<B, T, V><<<gb, kT, 0, s>>>(n, a.dinv, a.t, x, omega, sc, slot);
      }
      return;
    }
    const L& c = lv[l + 1];
    count_launches(2);
    k_residual<B, T, V><<<gr, kT, 0, s>>>(n, a.rowptr, a.colidx, a.val, x, r, a.t, sc, slot);
    k_restrict<B, T><<<blocks_for(a.ncoarse), kT, 0, s>>>(static_cast<int>(a.ncoarse), a.agg_ptr, a.agg_rows, a.t,
                                                          c.rc, sc, slot);
    run(lv, l + 1, c.rc, c.x, omega, sweeps, sc, slot, s);
    count_launches(3);
    k_prolong<B, T><<<gr, kT, 0, s>>>(n, a.agg, c.x, x, sc, slot);
    k_residual<B, T, V><<<gr, kT, 0, s>>>(n, a.rowptr, a.colidx, a.val, x, r, a.t, sc, slot);
    k_bj_axpy<B, T, V><<<gb, kT, 0, s>>>(n, a.dinv, a.t, x, omega, sc, slot);
  }
};

}  // namespace

void Amg::build(const std::vector<int32_t>& rowptr, const std::vector<int32_t>& colidx,
                const std::vector<int32_t>& diag, const std::vector<int32_t>& group, int bs, int max_levels,
                int min_rows) {
  levels_.clear();
  bs_ = bs;
  std::vector<int32_t> rp = rowptr, ci = colidx, dg = diag, grp = group;
  int64_t n = static_cast<int64_t>(rp.size()) - 1;
  for (int l = 0; l < max_levels; ++l) {
    Level L;
    L.nrows = n;
    L.nnzb = static_cast<int64_t>(ci.size());
    L.rowptr_o.upload(rp);
    L.colidx_o.upload(ci);
    L.diag_o.upload(dg);
    L.rowptr = L.rowptr_o.get();
    L.colidx = L.colidx_o.get();
    L.diag = L.diag_o.get();
    const bool last = (l + 1 == max_levels) || n <= min_rows;
    if (last) {
      levels_.push_back(std::move(L));
      break;
    }
    // greedy aggregation within groups
    std::vector<int32_t> agg(n, -1);
    int32_t na = 0;
    for (int64_t i = 0; i < n; ++i) {
      if (agg[i] != -1) continue;
      bool free_nb = true;
      for (int32_t k = rp[i]; k < rp[i + 1] && free_nb; ++k) {
        const int32_t j = ci[k];
        if (j != i && grp[j] == grp[i] && agg[j] != -1) free_nb = false;
      }
      if (!free_nb) continue;
      agg[i] = na;
      for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
        const int32_t j = ci[k];
        if (grp[j] == grp[i]) agg[j] = na;
      }
      ++na;
    }
    const std::vector<int32_t> agg1 = agg;
    for (int64_t i = 0; i < n; ++i) {
      if (agg[i] != -1) continue;
      for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
        const int32_t j = ci[k];
        if (j != i && grp[j] == grp[i] && agg1[j] != -1) {
          agg[i] = agg1[j];
          break;
        }
      }
    }
    for (int64_t i = 0; i < n; ++i)
      if (agg[i] == -1) agg[i] = na++;
    if (na >= 0.9 * n) {  // coarsening stalled: this level is the coarsest
      levels_.push_back(std::move(L));
      break;
    }
    // aggregate members (CSR)
    std::vector<int32_t> aptr(na + 1, 0), arows(n);
    for (int64_t i = 0; i < n; ++i) aptr[agg[i] + 1]++;
    for (int32_t a = 0; a < na; ++a) aptr[a + 1] += aptr[a];
    {
      std::vector<int32_t> fill(aptr.begin(), aptr.end() - 1);
      for (int64_t i = 0; i < n; ++i) arows[fill[agg[i]]++] = static_cast<int32_t>(i);
    }
    // coarse pattern
    std::vector<int32_t> crp(na + 1, 0), cci, cdg(na, -1), cgrp(na, 0);
    std::vector<int32_t> cols;
    for (int32_t a = 0; a < na; ++a) {
      cols.clear();
      for (int32_t q = aptr[a]; q < aptr[a + 1]; ++q) {
        const int32_t i = arows[q];
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) cols.push_back(agg[ci[k]]);
      }
      std::sort(cols.begin(), cols.end());
      cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
      for (int32_t c : cols) {
        if (c == a) cdg[a] = static_cast<int32_t>(cci.size());
        cci.push_back(c);
      }
      crp[a + 1] = static_cast<int32_t>(cci.size());
      cgrp[a] = grp[arows[aptr[a]]];
    }
    // fine block -> coarse block, grouped per coarse block in increasing fine order
    std::vector<int32_t> target(ci.size());
    for (int64_t i = 0; i < n; ++i) {
      const int32_t I = agg[i];
      for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
        const int32_t J = agg[ci[k]];
        auto b = cci.begin() + crp[I], e = cci.begin() + crp[I + 1];
        target[k] = static_cast<int32_t>(std::lower_bound(b, e, J) - cci.begin());
      }
    }
    std::vector<int32_t> gptr(cci.size() + 1, 0), gsrc(ci.size());
    for (size_t k = 0; k < ci.size(); ++k) gptr[target[k] + 1]++;
    for (size_t c = 0; c < cci.size(); ++c) gptr[c + 1] += gptr[c];
    {
      std::vector<int32_t> fill(gptr.begin(), gptr.end() - 1);
      for (size_t k = 0; k < ci.size(); ++k) gsrc[fill[target[k]]++] = static_cast<int32_t>(k);
    }
    L.agg.upload(agg);
    L.agg_ptr.upload(aptr);
    L.agg_rows.upload(arows);
    L.gal_ptr.upload(gptr);
    L.gal_src.upload(gsrc);
    levels_.push_back(std::move(L));
    rp = std::move(crp);
    ci = std::move(cci);
    dg = std::move(cdg);
    grp = std::move(cgrp);
    n = na;
  }
  // values and work vectors
  for (size_t l = 0; l < levels_.size(); ++l) {
    Level& L = levels_[l];
    const int64_t nv = L.nrows * bs_;
    if (l > 0) {
      L.val_o.resize(L.nnzb * bs_ * bs_);
      L.dinv_o.resize(L.nrows * bs_ * bs_);
      L.val = L.val_o.get();
      L.dinv = L.dinv_o.get();
    }
    L.x.resize(nv);
    L.t.resize(nv);
    L.rc.resize(nv);
  }
  cuda_check(cudaStreamSynchronize(cudaStreamLegacy), "multigrid set-up");
}

void Amg::setup(const double* fine_vals, const double* fine_dinv, const float* fine_vals32,
                const float* fine_dinv32, bool fp32, int* status, cudaStream_t s) {
  if (levels_.empty()) return;
  levels_[0].val = fine_vals;
  levels_[0].dinv = fine_dinv;
  levels_[0].val32 = fine_vals32;
  levels_[0].dinv32 = fine_dinv32;
  const int bs2 = bs_ * bs_;
  for (size_t l = 1; l < levels_.size(); ++l) {
    Level& f = levels_[l - 1];
    Level& c = levels_[l];
    const int64_t ne = c.nnzb * bs2;
    count_launches(1);
    k_galerkin<<<blocks_for(ne), kT, 0, s>>>(ne, bs2, f.gal_ptr.get(), f.gal_src.get(), f.val, c.val_o.get());
    Bsr A;
    A.nrows = static_cast<int>(c.nrows);
    A.bs = bs_;
    A.nnzb = c.nnzb;
    A.rowptr = c.rowptr;
    A.colidx = c.colidx;
    A.val = c.val_o.get();
    block_jacobi_setup(A, c.diag, c.dinv_o.get(), status, s);
  }
  if (fp32) {
    for (size_t l = 1; l < levels_.size(); ++l) {
      Level& c = levels_[l];
      if (c.val32_o.size() != c.val_o.size()) {
        c.val32_o.resize(c.val_o.size());
        c.dinv32_o.resize(c.dinv_o.size());
      }
      to_float(static_cast<int64_t>(c.val_o.size()), c.val_o.get(), c.val32_o.get(), s);
      to_float(static_cast<int64_t>(c.dinv_o.size()), c.dinv_o.get(), c.dinv32_o.get(), s);
      c.val32 = c.val32_o.get();
      c.dinv32 = c.dinv32_o.get();
    }
    for (auto& L : levels_)
      if (L.x32.size() != L.x.size()) {
        L.x32.resize(L.x.size());
        L.t32.resize(L.t.size());
        L.rc32.resize(L.rc.size());
      }
  }
}

template <class T>
void Amg::apply(const T* r, T* z, const double* sc, int done_slot, cudaStream_t s) const {
  constexpr bool f32 = std::is_same<T, float>::value;
  using V = T;
#define DC_AMG(B)                                                                                        \
  case B: {                                                                                              \
    std::vector<typename Cycle<B, T, V>::L> lv(levels_.size());                                          \
    for (size_t l = 0; l < levels_.size(); ++l) {                                                        \
      const Level& L = levels_[l];                                                                       \
      auto& o = lv[l];                                                                                   \
      o.nrows = L.nrows;                                                                                 \
      o.rowptr = L.rowptr;                                                                               \
      o.colidx = L.colidx;                                                                               \
      o.agg = L.agg.get();                                                                               \
      o.agg_ptr = L.agg_ptr.get();                                                                       \
      o.agg_rows = L.agg_rows.get();                                                                     \
      o.ncoarse = (l + 1 < levels_.size()) ? levels_[l + 1].nrows : 0;                                   \
      if constexpr (f32) {                                                                               \
        o.val = reinterpret_cast<const V*>(L.val32);                                                     \
        o.dinv = reinterpret_cast<const V*>(L.dinv32);                                                   \
        o.x = reinterpret_cast<T*>(L.x32.get());                                                         \
        o.t = reinterpret_cast<T*>(L.t32.get());                                                         \
        o.rc = reinterpret_cast<T*>(L.rc32.get());                                                       \
      } else {                                                                                           \
        o.val = reinterpret_cast<const V*>(L.val);                                                       \
        o.dinv = reinterpret_cast<const V*>(L.dinv);                                                     \
        o.x = reinterpret_cast<T*>(L.x.get());                                                           \
        o.t = reinterpret_cast<T*>(L.t.get());                                                           \
        o.rc = reinterpret_cast<T*>(L.rc.get());                                                         \
      }                                                                                                  \
    }                                                                                                    \
    Cycle<B, T, V>::run(lv, 0, r, z, static_cast<V>(omega), coarse_sweeps, sc, done_slot, s);            \
    break;                                                                                               \
  }
  switch (bs_) {
    DC_AMG(1) DC_AMG(2) DC_AMG(3) DC_AMG(4) DC_AMG(5) DC_AMG(6) DC_AMG(7) DC_AMG(8)
    default: throw std::runtime_error("multigrid: block size " + std::to_string(bs_) + " unsupported");
  }
#undef DC_AMG
}

template void Amg::apply<double>(const double*, double*, const double*, int, cudaStream_t) const;
template void Amg::apply<float>(const float*, float*, const double*, int, cudaStream_t) const;

}  // namespace dcgpu
