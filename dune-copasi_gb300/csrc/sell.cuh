// Sliced block-ELL ("SELL-32") layout of the BSR pattern, used for the single-precision
// Krylov operator.
//
// Block rows are taken in slices of 32 consecutive rows.  Slot k of a slice holds the k-th
// stored block of each of its 32 rows, zero padded up to the slice's longest row.  Entry
// (i, j) of slot k of lane r (row 32 s + r) sits at ((off[s] + k) * B*B + i*B + j) * 32 + r
// and the slot's block column at (off[s] + k) * 32 + r.  A warp computes one slice, one lane
// per block row: every value load of the warp is one contiguous 128-byte line, the column
// load too, against (32 / B) scattered B-value segments per load of the thread-per-row BSR
// kernel.  Padding slots point at the row itself and hold zeros.
#pragma once

#include <cstdint>

namespace dcgpu {

struct Sell {
  int nrows = 0;                  // block rows
  int bs = 1;
  int64_t nslices = 0;
  int64_t nslots = 0;             // total slots (each 32 lanes wide)
  const int64_t* off = nullptr;   // nslices + 1 slot offsets
  const int32_t* cols = nullptr;  // nslots * 32 block columns
};

#ifdef __CUDACC__
// y rows of slice `sl` for lane `lane`: acc[i] = sum over the lane's blocks of A(i, :) x.
// kCoherent reads x through L2 only (ld.global.cg), for kernels in which other blocks write x
// between grid-wide barriers; the operator itself is read-only and uses the read-only path.
template <int B, class T, class V, bool kCoherent = false>
__device__ __forceinline__ void sell_lane_rows(const Sell& S, int64_t sl, int lane, const V* __restrict__ val,
                                               const T* __restrict__ x, V (&acc)[B]) {
#pragma unroll
  for (int i = 0; i < B; ++i) acc[i] = V(0);
  const int64_t o0 = S.off[sl], o1 = S.off[sl + 1];
  const int32_t* __restrict__ cols = S.cols + o0 * 32 + lane;
  const V* __restrict__ v = val + o0 * (32 * B * B) + lane;
  const int w = static_cast<int>(o1 - o0);
  // slots in batches of U: the U column loads, then the U x gathers, are independent of
  // one another, so a lane has U (not one) dependent load chains in flight; the slice's
  // time is then a few L2 round trips instead of two per slot
  constexpr int U = B <= 2 ? 4 : 2;
  int k = 0;
  for (; k + U <= w; k += U) {
    int c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) c[u] = __ldg(cols + (k + u) * 32);
    V xv[U][B];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int j = 0; j < B; ++j) {
        const T* xp = x + static_cast<int64_t>(c[u]) * B + j;
        xv[u][j] = static_cast<V>(kCoherent ? __ldcg(xp) : *xp);
      }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const V* __restrict__ vk = v + static_cast<int64_t>(k + u) * (32 * B * B);
#pragma unroll
      for (int i = 0; i < B; ++i)
#pragma unroll
        for (int j = 0; j < B; ++j) acc[i] += __ldg(vk + (i * B + j) * 32) * xv[u][j];
    }
  }
  for (; k < w; ++k) {
    const int c = __ldg(cols + k * 32);
    V xv[B];
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const T* xp = x + static_cast<int64_t>(c) * B + j;
      xv[j] = static_cast<V>(kCoherent ? __ldcg(xp) : *xp);
    }
    const V* __restrict__ vk = v + static_cast<int64_t>(k) * (32 * B * B);
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
      for (int j = 0; j < B; ++j) acc[i] += __ldg(vk + (i * B + j) * 32) * xv[j];
  }
}
#endif

}  // namespace dcgpu
