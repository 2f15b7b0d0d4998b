// Lane-per-row products on an entry-interleaved SELL-32 layout, for the preconditioner
// kernels.
//
// The slot structure is that of sell.cuh (slices of 32 block rows, slot k of a slice holding
// the k-th stored block of each of its rows, zero padded; columns at (off[s] + k) * 32 + r).
// The values are interleaved by entry: entry e of the block of slot p and lane r sits at
// (p * B*B + e) * 32 + r, so a warp reading one entry of its 32 blocks reads one contiguous
// line (128 bytes in fp32) whatever the block size (the per-lane contiguous blocks of the
// Krylov operator need 16-byte vector loads, which a 5 x 5 block cannot use).
#pragma once

#include <cstdint>

#include "sell.cuh"

namespace dcgpu {

// acc[s] += sum over the lane's slots whose block column c passes use(c) of
// A_slot(s, :) x_c, with x_c produced by fetch(c, xv).  Padding slots hold zero blocks.
template <int B, class V, class Use, class Fetch>
__device__ __forceinline__ void sell_row_apply(const Sell& S, int64_t sl, int lane, const V* __restrict__ val,
                                               Use use, Fetch fetch, V (&acc)[B]) {
  const int64_t o0 = S.off[sl];
  const int w = static_cast<int>(S.off[sl + 1] - o0);
  const int32_t* __restrict__ cols = S.cols + o0 * 32 + lane;
  const V* __restrict__ v = val + o0 * 32 * (B * B) + lane;
#pragma unroll 2
  for (int k = 0; k < w; ++k) {
    const int32_t c = __ldg(cols + static_cast<int64_t>(k) * 32);
    if (!use(c)) continue;
    V xv[B];
    fetch(c, xv);
    const V* __restrict__ b = v + static_cast<int64_t>(k) * (32 * B * B);
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
      for (int j = 0; j < B; ++j) acc[i] += __ldg(b + (i * B + j) * 32) * xv[j];
  }
}

// warps of the launch and the slice of each, for grid-stride loops over slices
struct SliceLoop {
  int64_t first, stride;
  int lane;
  __device__ SliceLoop() {
    const int warps_per_block = blockDim.x / 32;
    first = static_cast<int64_t>(blockIdx.x) * warps_per_block + threadIdx.x / 32;
    stride = static_cast<int64_t>(gridDim.x) * warps_per_block;
    lane = threadIdx.x % 32;
  }
};

}  // namespace dcgpu
