// Sliced block-ELL ("SELL-32") layout of the BSR pattern, used for the single-precision
// Krylov operator.
//
// Block rows are taken in slices of 32 consecutive rows.  Slot k of a slice holds the k-th
// stored block of each of its 32 rows, zero padded up to the slice's longest row.  Slot
// position p = (off[s] + k) * 32 + r belongs to lane r (row 32 s + r); the slot's block
// column sits at cols[p], and entry e (row-major) of its B x B block at
// sell_value_index(p, e, B*B) = (off[s] + k) * 32 * B*B + e * 32 + r: the values are
// interleaved by entry, so when a warp (one slice, one lane per block row) reads entry e of
// its 32 blocks it reads one contiguous line (128 bytes in fp32) for every block size, and
// the column load of the warp is one 128-byte line as well.  Padding slots point at the row
// itself (row 0 past the last row) and hold zeros.
#pragma once

#include <cstdint>
#include <type_traits>

namespace dcgpu {

// index of entry e of the block at slot position p (bs2 = B*B values per block)
__host__ __device__ inline int64_t sell_value_index(int64_t p, int e, int bs2) {
  return (p >> 5) * 32 * bs2 + static_cast<int64_t>(e) * 32 + (p & 31);
}

struct Sell {
  int nrows = 0;                  // block rows
  int bs = 1;
  int64_t nslices = 0;
  int64_t nslots = 0;             // total slots (each 32 lanes wide)
  const int64_t* off = nullptr;   // nslices + 1 slot offsets
  const int32_t* cols = nullptr;  // nslots * 32 block columns
};

#ifdef __CUDACC__
// the N = B*B entries of one lane's block in the entry-interleaved layout (p: entry 0)
template <int N, class V>
__device__ __forceinline__ void load_block_interleaved(const V* __restrict__ p, V (&out)[N]) {
#pragma unroll
  for (int e = 0; e < N; ++e) out[e] = __ldg(p + e * 32);
}

// N consecutive values starting at p: 8- or 16-byte loads for fp32 runs of 2 or a multiple
// of 4 values (the callers' offsets are multiples of 8 / 16 bytes), else N loads.
// kCoherent reads through L2 only (ld.global.cg, for data that other blocks write inside
// the same launch), otherwise through the read-only path.
template <int N, bool kCoherent, class T>
__device__ __forceinline__ void load_block(const T* __restrict__ p, T (&out)[N]) {
  if constexpr (std::is_same_v<T, float> && N == 2) {
    const float2 q = kCoherent ? __ldcg(reinterpret_cast<const float2*>(p)) : __ldg(reinterpret_cast<const float2*>(p));
    out[0] = q.x;
    out[1] = q.y;
  } else if constexpr (std::is_same_v<T, float> && N % 4 == 0) {
#pragma unroll
    for (int j = 0; j < N; j += 4) {
      const float4 q = kCoherent ? __ldcg(reinterpret_cast<const float4*>(p + j))
                                 : __ldg(reinterpret_cast<const float4*>(p + j));
      out[j] = q.x;
      out[j + 1] = q.y;
      out[j + 2] = q.z;
      out[j + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) out[j] = kCoherent ? __ldcg(p + j) : __ldg(p + j);
  }
}

// y rows of slice `sl` for lane `lane`: acc[i] = sum over the lane's blocks of A(i, :) x.
// kCoherent reads x through L2 only, for kernels in which other blocks write x between
// grid-wide barriers; the operator itself is read-only and uses the read-only path.
template <int B, class T, class V, bool kCoherent = false>
__device__ __forceinline__ void sell_lane_rows(const Sell& S, int64_t sl, int lane, const V* __restrict__ val,
                                               const T* __restrict__ x, V (&acc)[B]) {
#pragma unroll
  for (int i = 0; i < B; ++i) acc[i] = V(0);
  const int64_t o0 = S.off[sl], o1 = S.off[sl + 1];
  const int32_t* __restrict__ cols = S.cols + o0 * 32 + lane;
  const V* __restrict__ v = val + o0 * 32 * (B * B) + lane;
  const int w = static_cast<int>(o1 - o0);
  // slots in batches of U: the U column loads, then the U x gathers, are independent of
  // one another, so a lane has U (not one) dependent load chains in flight, and the next
  // batch's column indices load while this batch's gathers are in flight
  constexpr int U = B <= 2 ? 4 : 2;
  int cn[U];
#pragma unroll
  for (int u = 0; u < U; ++u) cn[u] = u < w ? __ldg(cols + u * 32) : 0;
  int k = 0;
  for (; k + U <= w; k += U) {
    int c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      c[u] = cn[u];
      const int kn = k + U + u;
      cn[u] = kn < w ? __ldg(cols + kn * 32) : 0;
    }
    T xv[U][B];
#pragma unroll
    for (int u = 0; u < U; ++u) load_block<B, kCoherent>(x + static_cast<int64_t>(c[u]) * B, xv[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      V blk[B * B];
      load_block_interleaved<B * B>(v + static_cast<int64_t>(k + u) * (32 * B * B), blk);
#pragma unroll
      for (int i = 0; i < B; ++i)
#pragma unroll
        for (int j = 0; j < B; ++j) acc[i] += blk[i * B + j] * static_cast<V>(xv[u][j]);
    }
  }
  // the last w % U slots, whose columns are already in cn
#pragma unroll
  for (int u = 0; u < U - 1; ++u) {
    if (k + u >= w) break;
    T xv[B];
    load_block<B, kCoherent>(x + static_cast<int64_t>(cn[u]) * B, xv);
    V blk[B * B];
    load_block_interleaved<B * B>(v + static_cast<int64_t>(k + u) * (32 * B * B), blk);
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
      for (int j = 0; j < B; ++j) acc[i] += blk[i * B + j] * static_cast<V>(xv[j]);
  }
}
#endif

}  // namespace dcgpu
