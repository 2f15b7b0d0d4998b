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
// y rows of slice `sl` for lane `lane`: acc[i] = sum over the lane's blocks of A(i, :) x
template <int B, class T, class V>
__device__ __forceinline__ void sell_lane_rows(const Sell& S, int64_t sl, int lane, const V* __restrict__ val,
                                               const T* __restrict__ x, V (&acc)[B]) {
#pragma unroll
  for (int i = 0; i < B; ++i) acc[i] = V(0);
  const int64_t o0 = S.off[sl], o1 = S.off[sl + 1];
  const int32_t* __restrict__ cols = S.cols + o0 * 32 + lane;
  const V* __restrict__ v = val + o0 * (32 * B * B) + lane;
  const int w = static_cast<int>(o1 - o0);
#pragma unroll 2
  for (int k = 0; k < w; ++k) {
    const int c = __ldg(cols + k * 32);
    V xv[B];
#pragma unroll
    for (int j = 0; j < B; ++j) xv[j] = static_cast<V>(x[static_cast<int64_t>(c) * B + j]);
    const V* __restrict__ vk = v + static_cast<int64_t>(k) * (32 * B * B);
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
      for (int j = 0; j < B; ++j) acc[i] += __ldg(vk + (i * B + j) * 32) * xv[j];
  }
}
#endif

}  // namespace dcgpu
