#include "graph.hpp"

#include <climits>
#include <stdexcept>
#include <string>

#include "linalg.cuh"

namespace dcgpu {

namespace {

constexpr int kT = 256;

inline int grid_for_rows(int64_t n) {
  int64_t b = (n + kT - 1) / kT;
  return static_cast<int>(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

// Row priority: the 32-bit finaliser of MurmurHash3 (public domain, A. Appleby) applied to
// the row index plus a fixed offset; ties are broken by the index.
__device__ __forceinline__ uint32_t row_priority(uint32_t i) {
  uint32_t h = i + 0x2545F491u;
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}
__device__ __forceinline__ bool beats(uint32_t pj, int64_t j, uint32_t pi, int64_t i) {
  return pj > pi || (pj == pi && j > i);
}
__device__ __forceinline__ bool same_group(const int32_t* group, int64_t i, int64_t j) {
  return group == nullptr || group[i] == group[j];
}

// ---------------------------------------------------------------- prefix sums
constexpr int kScanT = 256, kScanPer = 8, kTile = kScanT * kScanPer;

// exclusive scan of each tile of kTile entries; tile_sums[b] = the tile's total
__global__ void __launch_bounds__(kScanT) k_scan_tiles(const int32_t* __restrict__ in, int32_t* __restrict__ out,
                                                       int32_t* __restrict__ tile_sums, int64_t n) {
  __shared__ int32_t sh[kTile];
  __shared__ int32_t warp_tot[kScanT / 32];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kTile;
  for (int q = threadIdx.x; q < kTile; q += kScanT) {
    const int64_t g = base + q;
    sh[q] = g < n ? in[g] : 0;
  }
  __syncthreads();
  int32_t v[kScanPer];
  int32_t sum = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; ++j) {
    v[j] = sh[threadIdx.x * kScanPer + j];
    sum += v[j];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t x = sum;  // inclusive scan of the thread sums within the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t t = lane < kScanT / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kScanT / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  int32_t run = x - sum + (w > 0 ? warp_tot[w - 1] : 0);
#pragma unroll
  for (int j = 0; j < kScanPer; ++j) {
    sh[threadIdx.x * kScanPer + j] = run;
    run += v[j];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kTile; q += kScanT) {
    const int64_t g = base + q;
    if (g < n) out[g] = sh[q];
  }
  if (threadIdx.x == kScanT - 1) tile_sums[blockIdx.x] = run;
}

__global__ void k_scan_add(int32_t* __restrict__ out, const int32_t* __restrict__ offs, int64_t n, int64_t ntiles) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < n; g += stride)
    out[g] += offs[g / kTile];
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = offs[ntiles];
}

__global__ void k_set_total(int32_t* out, int64_t n, const int32_t* tile_sum) { out[n] = tile_sum[0]; }

// ---------------------------------------------------------------- colouring
// One Jones-Plassmann round.  when[i] < 0: uncoloured; when[i] = r: coloured in round r.
// A row coloured in this round (when == r) still counts as uncoloured for its neighbours,
// so every decision depends on the state at the start of the round only.
__global__ void k_jp_round(int64_t n, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                           int32_t* __restrict__ colour, int32_t* __restrict__ when, int r, int32_t* remaining,
                           int32_t* max_colour) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (when[i] >= 0) continue;
    const uint32_t pi = row_priority(static_cast<uint32_t>(i));
    bool top = true;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1] && top; ++k) {
      const int32_t j = colidx[k];
      if (j == i) continue;
      const int32_t wj = when[j];
      if ((wj < 0 || wj == r) && beats(row_priority(static_cast<uint32_t>(j)), j, pi, i)) top = false;
    }
    if (!top) {
      atomicAdd(remaining, 1);
      continue;
    }
    // smallest colour that no neighbour coloured in an earlier round has
    int c = 0;
    for (;;) {
      unsigned long long used = 0ull;  // colours c .. c + 63
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
        const int32_t j = colidx[k];
        if (j == i) continue;
        const int32_t wj = when[j];
        if (wj >= 0 && wj < r) {
          const int d = colour[j] - c;
          if (d >= 0 && d < 64) used |= 1ull << d;
        }
      }
      if (used != ~0ull) {
        c += __ffsll(static_cast<long long>(~used)) - 1;
        break;
      }
      c += 64;
    }
    colour[i] = c;
    when[i] = r;
    atomicMax(max_colour, c);
  }
}

__global__ void k_flag_eq(int64_t n, const int32_t* __restrict__ key, int32_t v, int32_t* __restrict__ flag) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    flag[i] = key[i] == v ? 1 : 0;
}

__global__ void k_scatter_flagged(int64_t n, const int32_t* __restrict__ key, int32_t v,
                                  const int32_t* __restrict__ pos, int64_t base, int32_t* __restrict__ perm) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    if (key[i] == v) perm[base + pos[i]] = static_cast<int32_t>(i);
}

// ---------------------------------------------------------------- MIS-k aggregation
// state: 0 outside the set, 1 undecided, 2 in the set (a root)
__device__ __forceinline__ unsigned long long mis_tuple(int32_t state, int64_t i) {
  return (static_cast<unsigned long long>(state) << 62) |
         (static_cast<unsigned long long>(row_priority(static_cast<uint32_t>(i)) >> 1) << 31) |
         static_cast<unsigned long long>(i);
}

__global__ void k_mis_tuples(int64_t n, const int32_t* __restrict__ state, unsigned long long* __restrict__ t) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    t[i] = mis_tuple(state[i], i);
}

// tout[i] = max of tin over i and its neighbours in the same group
__global__ void k_mis_spread(DeviceGraph g, const unsigned long long* __restrict__ tin,
                             unsigned long long* __restrict__ tout) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < g.n; i += stride) {
    unsigned long long m = tin[i];
    for (int32_t k = g.rowptr[i]; k < g.rowptr[i + 1]; ++k) {
      const int32_t j = g.colidx[k];
      if (j != i && same_group(g.group, i, j) && tin[j] > m) m = tin[j];
    }
    tout[i] = m;
  }
}

__global__ void k_mis_decide(int64_t n, const unsigned long long* __restrict__ t, int32_t* __restrict__ state,
                             int32_t* remaining) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (state[i] != 1) continue;
    if (t[i] == mis_tuple(1, i)) state[i] = 2;
    else if ((t[i] >> 62) == 2ull) state[i] = 0;
    else atomicAdd(remaining, 1);
  }
}

__global__ void k_root_flags(int64_t n, const int32_t* __restrict__ state, int32_t* __restrict__ flag) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    flag[i] = state[i] == 2 ? 1 : 0;
}

// roots: their own aggregate; rows next to a root: the highest-priority adjacent root's
__global__ void k_agg_roots(DeviceGraph g, const int32_t* __restrict__ state, const int32_t* __restrict__ root_id,
                            int32_t* __restrict__ agg1) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < g.n; i += stride) {
    if (state[i] == 2) {
      agg1[i] = root_id[i];
      continue;
    }
    int64_t best = -1;
    uint32_t pb = 0;
    for (int32_t k = g.rowptr[i]; k < g.rowptr[i + 1]; ++k) {
      const int32_t j = g.colidx[k];
      if (j == i || !same_group(g.group, i, j) || state[j] != 2) continue;
      const uint32_t pj = row_priority(static_cast<uint32_t>(j));
      if (best < 0 || beats(pj, j, pb, best)) {
        best = j;
        pb = pj;
      }
    }
    agg1[i] = best >= 0 ? root_id[best] : -1;
  }
}

// rows without an adjacent root: the aggregate of the highest-priority neighbour that has one
__global__ void k_agg_rest(DeviceGraph g, const int32_t* __restrict__ agg1, int32_t* __restrict__ agg,
                           int32_t* unassigned) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < g.n; i += stride) {
    if (agg1[i] >= 0) {
      agg[i] = agg1[i];
      continue;
    }
    int64_t best = -1;
    uint32_t pb = 0;
    for (int32_t k = g.rowptr[i]; k < g.rowptr[i + 1]; ++k) {
      const int32_t j = g.colidx[k];
      if (j == i || !same_group(g.group, i, j) || agg1[j] < 0) continue;
      const uint32_t pj = row_priority(static_cast<uint32_t>(j));
      if (best < 0 || beats(pj, j, pb, best)) {
        best = j;
        pb = pj;
      }
    }
    agg[i] = best >= 0 ? agg1[best] : -1;
    if (best < 0) atomicAdd(unassigned, 1);
  }
}

// ---------------------------------------------------------------- coarse structure
__global__ void k_count_keys(int64_t n, const int32_t* __restrict__ key, int32_t* __restrict__ cnt) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    atomicAdd(&cnt[key[i]], 1);
}

// members of each aggregate in slots of arbitrary order (sorted afterwards)
__global__ void k_place_members(int64_t n, const int32_t* __restrict__ agg, const int32_t* __restrict__ ptr,
                                int32_t* __restrict__ cursor, int32_t* __restrict__ rows) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t a = agg[i];
    rows[ptr[a] + atomicAdd(&cursor[a], 1)] = static_cast<int32_t>(i);
  }
}

__device__ void insertion_sort(int32_t* v, int32_t len) {
  for (int32_t a = 1; a < len; ++a) {
    const int32_t x = v[a];
    int32_t b = a - 1;
    while (b >= 0 && v[b] > x) {
      v[b + 1] = v[b];
      --b;
    }
    v[b + 1] = x;
  }
}

// sorts each aggregate's members; nnz_of[a] = the members' stored blocks in the fine graph
__global__ void k_sort_members(int64_t na, const int32_t* __restrict__ ptr, int32_t* __restrict__ rows,
                               const int32_t* __restrict__ rowptr, int32_t* __restrict__ nnz_of) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; a < na; a += stride) {
    insertion_sort(rows + ptr[a], ptr[a + 1] - ptr[a]);
    int32_t z = 0;
    for (int32_t q = ptr[a]; q < ptr[a + 1]; ++q) z += rowptr[rows[q] + 1] - rowptr[rows[q]];
    nnz_of[a] = z;
  }
}

// the sorted distinct aggregates adjacent to aggregate I, in scratch[soff[I]...]; ucount[I]
__global__ void k_coarse_columns(int64_t na, const int32_t* __restrict__ ptr, const int32_t* __restrict__ rows,
                                 const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                                 const int32_t* __restrict__ agg, const int32_t* __restrict__ soff,
                                 int32_t* __restrict__ scratch, int32_t* __restrict__ ucount) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t I = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; I < na; I += stride) {
    int32_t* u = scratch + soff[I];
    int32_t nu = 0;
    for (int32_t q = ptr[I]; q < ptr[I + 1]; ++q) {
      const int32_t i = rows[q];
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
        const int32_t J = agg[colidx[k]];
        int32_t lo = 0, hi = nu;  // first position with u[pos] >= J
        while (lo < hi) {
          const int32_t mid = (lo + hi) >> 1;
          if (u[mid] < J) lo = mid + 1;
          else hi = mid;
        }
        if (lo < nu && u[lo] == J) continue;
        for (int32_t b = nu; b > lo; --b) u[b] = u[b - 1];
        u[lo] = J;
        ++nu;
      }
    }
    ucount[I] = nu;
  }
}

__global__ void k_coarse_fill(int64_t na, const int32_t* __restrict__ soff, const int32_t* __restrict__ scratch,
                              const int32_t* __restrict__ crp, int32_t* __restrict__ cci, int32_t* __restrict__ cdg,
                              const int32_t* __restrict__ ptr, const int32_t* __restrict__ rows,
                              const int32_t* __restrict__ fgroup, int32_t* __restrict__ cgroup, int32_t* missing) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t I = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; I < na; I += stride) {
    const int32_t* u = scratch + soff[I];
    int32_t d = -1;
    for (int32_t q = 0; q < crp[I + 1] - crp[I]; ++q) {
      cci[crp[I] + q] = u[q];
      if (u[q] == I) d = crp[I] + q;
    }
    cdg[I] = d;
    if (d < 0) atomicAdd(missing, 1);
    cgroup[I] = fgroup ? fgroup[rows[ptr[I]]] : 0;
  }
}

// pass 0: count the fine blocks of every coarse block; pass 1: list them (ascending fine
// block index: members ascend, and so do the blocks of a row)
template <int PASS>
__global__ void k_galerkin_lists(int64_t na, const int32_t* __restrict__ ptr, const int32_t* __restrict__ rows,
                                 const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                                 const int32_t* __restrict__ agg, const int32_t* __restrict__ crp,
                                 const int32_t* __restrict__ cci, int32_t* __restrict__ cnt,
                                 const int32_t* __restrict__ gptr, int32_t* __restrict__ gsrc) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t I = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; I < na; I += stride) {
    for (int32_t q = ptr[I]; q < ptr[I + 1]; ++q) {
      const int32_t i = rows[q];
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
        const int32_t J = agg[colidx[k]];
        int32_t lo = crp[I], hi = crp[I + 1];
        while (lo < hi) {
          const int32_t mid = (lo + hi) >> 1;
          if (cci[mid] < J) lo = mid + 1;
          else hi = mid;
        }
        if (PASS == 0) ++cnt[lo];
        else gsrc[gptr[lo] + cnt[lo]++] = k;
      }
    }
  }
}

// ---------------------------------------------------------------- SELL-32 layout
__global__ void k_slice_width(int64_t nslices, int64_t nrows, const int32_t* __restrict__ rowptr,
                              int32_t* __restrict__ width) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t sl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; sl < nslices; sl += stride) {
    int32_t w = 0;
    for (int64_t i = sl * 32; i < sl * 32 + 32 && i < nrows; ++i) w = max(w, rowptr[i + 1] - rowptr[i]);
    width[sl] = w;
  }
}

__global__ void k_widen(int64_t n, const int32_t* __restrict__ in, int64_t* __restrict__ out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i <= n; i += stride) out[i] = in[i];
}

// thread per (slice, lane): the lane's slots, padding pointing at the row itself (row 0
// past the last row)
__global__ void k_sell_fill(int64_t nslices, int64_t nrows, const int32_t* __restrict__ rowptr,
                            const int32_t* __restrict__ colidx, const int64_t* __restrict__ off,
                            int32_t* __restrict__ cols, int32_t* __restrict__ bpos) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < nslices * 32; t += stride) {
    const int64_t sl = t / 32, i = t;
    const int lane = static_cast<int>(t % 32);
    const int32_t len = i < nrows ? rowptr[i + 1] - rowptr[i] : 0;
    for (int64_t k = 0; k < off[sl + 1] - off[sl]; ++k) {
      const int64_t p = (off[sl] + k) * 32 + lane;
      if (k < len) {
        cols[p] = colidx[rowptr[i] + k];
        bpos[p] = static_cast<int32_t>(rowptr[i] + k);
      } else {
        cols[p] = i < nrows ? static_cast<int32_t>(i) : 0;
        bpos[p] = -1;
      }
    }
  }
}

// entry-interleaved values: out[(slot * bs2 + e) * 32 + lane] (sellrow.cuh)
template <class V>
__global__ void k_sell_values(int64_t nvals, int bs2, const int32_t* __restrict__ bpos, const double* __restrict__ bsr,
                              V* __restrict__ out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < nvals; t += stride) {
    const int64_t lane = t % 32, q = t / 32;
    const int64_t slot = q / bs2;
    const int e = static_cast<int>(q % bs2);
    const int32_t b = bpos[slot * 32 + lane];
    out[t] = b >= 0 ? static_cast<V>(bsr[static_cast<int64_t>(b) * bs2 + e]) : V(0);
  }
}

int32_t read_int(const int32_t* d, cudaStream_t s) {
  int32_t h = 0;
  cuda_check(cudaMemcpyAsync(&h, d, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "graph set-up read");
  cuda_check(cudaStreamSynchronize(s), "graph set-up");
  return h;
}

}  // namespace

void sell_structure(int64_t nrows, const int32_t* rowptr, const int32_t* colidx, SellStructure* out, cudaStream_t s) {
  SellStructure& S = *out;
  S.nrows = nrows;
  S.nslices = (nrows + 31) / 32;
  DeviceBuffer<int32_t> width(static_cast<size_t>(S.nslices)), off32(static_cast<size_t>(S.nslices) + 1);
  count_launches(1);
  k_slice_width<<<grid_for_rows(S.nslices), kT, 0, s>>>(S.nslices, nrows, rowptr, width.get());
  S.nslots = exclusive_scan(width.get(), off32.get(), S.nslices, s);
  S.off.resize(static_cast<size_t>(S.nslices) + 1);
  S.cols.resize(static_cast<size_t>(S.nslots) * 32);
  S.bpos.resize(static_cast<size_t>(S.nslots) * 32);
  count_launches(2);
  k_widen<<<grid_for_rows(S.nslices + 1), kT, 0, s>>>(S.nslices, off32.get(), S.off.get());
  k_sell_fill<<<grid_for_rows(S.nslices * 32), kT, 0, s>>>(S.nslices, nrows, rowptr, colidx, S.off.get(), S.cols.get(),
                                                           S.bpos.get());
  cuda_check(cudaStreamSynchronize(s), "SELL layout");
}

void sell_values(const SellStructure& S, int bs, const double* bsr, double* out, cudaStream_t s) {
  const int64_t nv = S.nslots * 32 * bs * bs;
  if (nv == 0) return;
  count_launches(1);
  k_sell_values<double><<<grid_for_rows(nv), kT, 0, s>>>(nv, bs * bs, S.bpos.get(), bsr, out);
}
void sell_values(const SellStructure& S, int bs, const double* bsr, float* out, cudaStream_t s) {
  const int64_t nv = S.nslots * 32 * bs * bs;
  if (nv == 0) return;
  count_launches(1);
  k_sell_values<float><<<grid_for_rows(nv), kT, 0, s>>>(nv, bs * bs, S.bpos.get(), bsr, out);
}

int64_t exclusive_scan(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s) {
  if (n <= 0) {
    cuda_check(cudaMemsetAsync(out, 0, sizeof(int32_t), s), "scan");
    return 0;
  }
  const int64_t ntiles = (n + kTile - 1) / kTile;
  DeviceBuffer<int32_t> sums(static_cast<size_t>(ntiles));
  count_launches(1);
  k_scan_tiles<<<static_cast<unsigned>(ntiles), kScanT, 0, s>>>(in, out, sums.get(), n);
  if (ntiles == 1) {
    count_launches(1);
    k_set_total<<<1, 1, 0, s>>>(out, n, sums.get());
  } else {
    DeviceBuffer<int32_t> offs(static_cast<size_t>(ntiles) + 1);
    exclusive_scan(sums.get(), offs.get(), ntiles, s);
    count_launches(1);
    k_scan_add<<<grid_for_rows(n), kT, 0, s>>>(out, offs.get(), n, ntiles);
    cuda_check(cudaStreamSynchronize(s), "scan");
  }
  return read_int(out + n, s);
}

int color_rows(const DeviceGraph& g, int32_t* colour, cudaStream_t s) {
  if (g.n <= 0) return 0;
  DeviceBuffer<int32_t> when(static_cast<size_t>(g.n)), counters(2);
  cuda_check(cudaMemsetAsync(when.get(), 0xff, g.n * sizeof(int32_t), s), "colour");
  cuda_check(cudaMemsetAsync(counters.get(), 0, 2 * sizeof(int32_t), s), "colour");
  // every round colours at least the uncoloured row of highest priority
  for (int r = 0;; ++r) {
    if (r > g.n) throw std::runtime_error("colouring did not finish");
    cuda_check(cudaMemsetAsync(counters.get(), 0, sizeof(int32_t), s), "colour");
    count_launches(1);
    k_jp_round<<<grid_for_rows(g.n), kT, 0, s>>>(g.n, g.rowptr, g.colidx, colour, when.get(), r, counters.get(),
                                                 counters.get() + 1);
    if (read_int(counters.get(), s) == 0) break;
  }
  return read_int(counters.get() + 1, s) + 1;
}

void order_by_color(int64_t n, const int32_t* colour, int ncolours, int32_t* perm, std::vector<int64_t>* offsets,
                    cudaStream_t s) {
  offsets->assign(static_cast<size_t>(ncolours) + 1, 0);
  if (n <= 0) return;
  DeviceBuffer<int32_t> flag(static_cast<size_t>(n)), pos(static_cast<size_t>(n) + 1);
  int64_t base = 0;
  for (int c = 0; c < ncolours; ++c) {
    count_launches(1);
    k_flag_eq<<<grid_for_rows(n), kT, 0, s>>>(n, colour, c, flag.get());
    const int64_t cnt = exclusive_scan(flag.get(), pos.get(), n, s);
    count_launches(1);
    k_scatter_flagged<<<grid_for_rows(n), kT, 0, s>>>(n, colour, c, pos.get(), base, perm);
    base += cnt;
    (*offsets)[c + 1] = base;
  }
  cuda_check(cudaStreamSynchronize(s), "colour order");
}

int64_t aggregate_mis(const DeviceGraph& g, int k, int32_t* agg, cudaStream_t s) {
  if (k != 1 && k != 2) throw std::runtime_error("aggregation: MIS distance must be 1 or 2");
  if (g.n <= 0) return 0;
  if (g.n >= (int64_t(1) << 31)) throw std::runtime_error("aggregation: too many rows");
  const size_t n = static_cast<size_t>(g.n);
  DeviceBuffer<int32_t> state(n), counter(1);
  DeviceBuffer<unsigned long long> ta(n), tb(n);
  {
    std::vector<int32_t> ones(n, 1);
    state.upload(ones);
  }
  for (int round = 0;; ++round) {
    if (round > g.n) throw std::runtime_error("aggregation: independent set did not finish");
    cuda_check(cudaMemsetAsync(counter.get(), 0, sizeof(int32_t), s), "aggregation");
    count_launches(2 + k);
    k_mis_tuples<<<grid_for_rows(g.n), kT, 0, s>>>(g.n, state.get(), ta.get());
    k_mis_spread<<<grid_for_rows(g.n), kT, 0, s>>>(g, ta.get(), tb.get());
    const unsigned long long* t = tb.get();
    if (k == 2) {
      k_mis_spread<<<grid_for_rows(g.n), kT, 0, s>>>(g, tb.get(), ta.get());
      t = ta.get();
    }
    k_mis_decide<<<grid_for_rows(g.n), kT, 0, s>>>(g.n, t, state.get(), counter.get());
    if (read_int(counter.get(), s) == 0) break;
  }
  DeviceBuffer<int32_t> flag(n), rid(n + 1), agg1(n);
  count_launches(1);
  k_root_flags<<<grid_for_rows(g.n), kT, 0, s>>>(g.n, state.get(), flag.get());
  const int64_t na = exclusive_scan(flag.get(), rid.get(), g.n, s);
  cuda_check(cudaMemsetAsync(counter.get(), 0, sizeof(int32_t), s), "aggregation");
  count_launches(2);
  k_agg_roots<<<grid_for_rows(g.n), kT, 0, s>>>(g, state.get(), rid.get(), agg1.get());
  k_agg_rest<<<grid_for_rows(g.n), kT, 0, s>>>(g, agg1.get(), agg, counter.get());
  if (read_int(counter.get(), s) != 0) throw std::runtime_error("aggregation left rows without an aggregate");
  return na;
}

void coarse_structure(const DeviceGraph& fine, const int32_t* agg, int64_t na, CoarseStructure* out, cudaStream_t s) {
  CoarseStructure& c = *out;
  const size_t nf = static_cast<size_t>(fine.n);
  c.n = na;
  DeviceBuffer<int32_t> cnt(static_cast<size_t>(na)), cursor(static_cast<size_t>(na)), nnz_of(static_cast<size_t>(na)),
      soff(static_cast<size_t>(na) + 1), ucount(static_cast<size_t>(na)), counter(1);
  c.agg_ptr.resize(static_cast<size_t>(na) + 1);
  c.agg_rows.resize(nf);
  cuda_check(cudaMemsetAsync(cnt.get(), 0, na * sizeof(int32_t), s), "coarse");
  cuda_check(cudaMemsetAsync(cursor.get(), 0, na * sizeof(int32_t), s), "coarse");
  count_launches(1);
  k_count_keys<<<grid_for_rows(fine.n), kT, 0, s>>>(fine.n, agg, cnt.get());
  exclusive_scan(cnt.get(), c.agg_ptr.get(), na, s);
  count_launches(2);
  k_place_members<<<grid_for_rows(fine.n), kT, 0, s>>>(fine.n, agg, c.agg_ptr.get(), cursor.get(), c.agg_rows.get());
  k_sort_members<<<grid_for_rows(na), kT, 0, s>>>(na, c.agg_ptr.get(), c.agg_rows.get(), fine.rowptr, nnz_of.get());
  const int64_t scratch_n = exclusive_scan(nnz_of.get(), soff.get(), na, s);
  DeviceBuffer<int32_t> scratch(static_cast<size_t>(scratch_n));
  count_launches(1);
  k_coarse_columns<<<grid_for_rows(na), kT, 0, s>>>(na, c.agg_ptr.get(), c.agg_rows.get(), fine.rowptr, fine.colidx,
                                                    agg, soff.get(), scratch.get(), ucount.get());
  c.rowptr.resize(static_cast<size_t>(na) + 1);
  c.nnzb = exclusive_scan(ucount.get(), c.rowptr.get(), na, s);
  c.colidx.resize(static_cast<size_t>(c.nnzb));
  c.diag.resize(static_cast<size_t>(na));
  c.group.resize(static_cast<size_t>(na));
  cuda_check(cudaMemsetAsync(counter.get(), 0, sizeof(int32_t), s), "coarse");
  count_launches(1);
  k_coarse_fill<<<grid_for_rows(na), kT, 0, s>>>(na, soff.get(), scratch.get(), c.rowptr.get(), c.colidx.get(),
                                                 c.diag.get(), c.agg_ptr.get(), c.agg_rows.get(), fine.group,
                                                 c.group.get(), counter.get());
  if (read_int(counter.get(), s) != 0) throw std::runtime_error("coarse level: a row without its diagonal block");
  // Galerkin lists
  DeviceBuffer<int32_t> gcnt(static_cast<size_t>(c.nnzb));
  cuda_check(cudaMemsetAsync(gcnt.get(), 0, c.nnzb * sizeof(int32_t), s), "coarse");
  count_launches(1);
  k_galerkin_lists<0><<<grid_for_rows(na), kT, 0, s>>>(na, c.agg_ptr.get(), c.agg_rows.get(), fine.rowptr,
                                                       fine.colidx, agg, c.rowptr.get(), c.colidx.get(), gcnt.get(),
                                                       nullptr, nullptr);
  c.gal_ptr.resize(static_cast<size_t>(c.nnzb) + 1);
  const int64_t total = exclusive_scan(gcnt.get(), c.gal_ptr.get(), c.nnzb, s);
  c.gal_src.resize(static_cast<size_t>(total));
  cuda_check(cudaMemsetAsync(gcnt.get(), 0, c.nnzb * sizeof(int32_t), s), "coarse");
  count_launches(1);
  k_galerkin_lists<1><<<grid_for_rows(na), kT, 0, s>>>(na, c.agg_ptr.get(), c.agg_rows.get(), fine.rowptr,
                                                       fine.colidx, agg, c.rowptr.get(), c.colidx.get(), gcnt.get(),
                                                       c.gal_ptr.get(), c.gal_src.get());
  cuda_check(cudaStreamSynchronize(s), "coarse level");
}

}  // namespace dcgpu
