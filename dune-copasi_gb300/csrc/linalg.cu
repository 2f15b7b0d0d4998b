#include "linalg.cuh"

#include <atomic>
#include <stdexcept>
#include <string>

namespace dcgpu {

namespace {

// ---------------------------------------------------------------- reductions
// Each thread accumulates a grid-strided slice in a fixed order, the block reduces with a
// fixed shuffle tree, and the last block to finish sums the per-block partials in index
// order.  The result is bitwise reproducible for a given n.

template <int NSUM>
__device__ __forceinline__ void block_sum(double (&acc)[NSUM], double (*sh)[kReduceThreads / 32]) {
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
      for (int w = 0; w < kReduceThreads / 32; ++w) v += sh[k][w];
      acc[k] = v;
    }
  }
}

template <int NSUM, class Body, class Fin>
__global__ void __launch_bounds__(kReduceThreads) k_reduce(int64_t n, Body body, Fin fin, ReduceScratch rs) {
  __shared__ double sh[NSUM][kReduceThreads / 32];
  __shared__ bool last;
  double acc[NSUM];
#pragma unroll
  for (int k = 0; k < NSUM; ++k) acc[k] = 0.0;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    body(i, acc);
  block_sum<NSUM>(acc, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NSUM; ++k) rs.partial[blockIdx.x * 4 + k] = acc[k];
    __threadfence();
    const unsigned prev = atomicAdd(rs.counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double tot[NSUM];
#pragma unroll
  for (int k = 0; k < NSUM; ++k) tot[k] = 0.0;
  for (int b = threadIdx.x; b < static_cast<int>(gridDim.x); b += blockDim.x)
#pragma unroll
    for (int k = 0; k < NSUM; ++k) tot[k] += __ldcg(&rs.partial[b * 4 + k]);
  __syncthreads();
  block_sum<NSUM>(tot, sh);
  if (threadIdx.x == 0) {
    fin(tot);
    *rs.counter = 0u;
  }
}

template <int NSUM, class Body, class Fin>
void reduce(int64_t n, Body body, Fin fin, ReduceScratch rs, cudaStream_t s) {
  count_launches(1);
  k_reduce<NSUM><<<kReduceBlocks, kReduceThreads, 0, s>>>(n, body, fin, rs);
}

struct DotBody {
  const double* x;
  const double* y;
  __device__ void operator()(int64_t i, double (&acc)[1]) const { acc[0] += x[i] * y[i]; }
};
struct StoreFin {
  double* out;
  __device__ void operator()(const double (&t)[1]) const { *out = t[0]; }
};

// ---------------------------------------------------------------- SpMV
// one thread per scalar row of the BSR matrix; the bs values of a block row segment
// are contiguous, neighbouring threads read neighbouring segments

template <int B, class V, class X>
__global__ void __launch_bounds__(256) k_spmv(int nrows, const int32_t* __restrict__ rowptr,
                                              const int32_t* __restrict__ colidx, const V* __restrict__ val,
                                              const X* __restrict__ x, X* __restrict__ y,
                                              const X* __restrict__ b, const double alpha,
                                              const int accumulate) {
  const int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (row >= static_cast<int64_t>(nrows) * B) return;
  const int br = static_cast<int>(row / B), i = static_cast<int>(row % B);
  // accumulate in the value type: fp64 for the fp64 operator, fp32 for the fp32 copy
  V acc = V(0);
  const int k0 = rowptr[br], k1 = rowptr[br + 1];
  for (int k = k0; k < k1; ++k) {
    const int c = colidx[k];
    const V* blk = val + static_cast<int64_t>(k) * B * B + i * B;
    const X* xc = x + static_cast<int64_t>(c) * B;
#pragma unroll
    for (int j = 0; j < B; ++j) acc += blk[j] * static_cast<V>(xc[j]);
  }
  if (accumulate) y[row] = static_cast<X>(static_cast<double>(y[row]) + alpha * static_cast<double>(acc));
  else if (b) y[row] = static_cast<X>(static_cast<double>(b[row]) - acc);
  else y[row] = static_cast<X>(acc);
}

template <class V, class X>
void spmv_dispatch(const Bsr& A, const V* val, const X* x, X* y, const X* b, cudaStream_t s,
                   double alpha = 1.0, int accumulate = 0) {
  const int64_t n = static_cast<int64_t>(A.nrows) * A.bs;
  if (n == 0) return;
  const int threads = 256;
  const int blocks = static_cast<int>((n + threads - 1) / threads);
  count_launches(1);
#define DC_SPMV(B) \
  case B: k_spmv<B, V, X><<<blocks, threads, 0, s>>>(A.nrows, A.rowptr, A.colidx, val, x, y, b, alpha, accumulate); return;
  switch (A.bs) {
    DC_SPMV(1) DC_SPMV(2) DC_SPMV(3) DC_SPMV(4) DC_SPMV(5) DC_SPMV(6) DC_SPMV(7) DC_SPMV(8)
    default: throw std::runtime_error("spmv: block size " + std::to_string(A.bs) + " unsupported");
  }
#undef DC_SPMV
}

// ---------------------------------------------------------------- block Jacobi

template <int B>
__global__ void k_bj_setup(int nrows, const int32_t* diag, const double* val, double* dinv, int* status,
                           float* dinv32) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  double a[B][B], inv[B][B];
  const double* blk = val + static_cast<int64_t>(diag[r]) * B * B;
#pragma unroll
  for (int i = 0; i < B; ++i)
#pragma unroll
    for (int j = 0; j < B; ++j) {
      a[i][j] = blk[i * B + j];
      inv[i][j] = (i == j) ? 1.0 : 0.0;
    }
  // Gauss-Jordan with partial pivoting
#pragma unroll
  for (int c = 0; c < B; ++c) {
    int piv = c;
    double best = fabs(a[c][c]);
#pragma unroll
    for (int i = c + 1; i < B; ++i)
      if (fabs(a[i][c]) > best) { best = fabs(a[i][c]); piv = i; }
    if (best == 0.0 || !isfinite(best)) { atomicExch(status, 1); return; }
    if (piv != c) {
#pragma unroll
      for (int j = 0; j < B; ++j) {
        double t = a[c][j]; a[c][j] = a[piv][j]; a[piv][j] = t;
        t = inv[c][j]; inv[c][j] = inv[piv][j]; inv[piv][j] = t;
      }
    }
    const double d = 1.0 / a[c][c];
#pragma unroll
    for (int j = 0; j < B; ++j) { a[c][j] *= d; inv[c][j] *= d; }
#pragma unroll
    for (int i = 0; i < B; ++i) {
      if (i == c) continue;
      const double f = a[i][c];
#pragma unroll
      for (int j = 0; j < B; ++j) { a[i][j] -= f * a[c][j]; inv[i][j] -= f * inv[c][j]; }
    }
  }
  double* o = dinv + static_cast<int64_t>(r) * B * B;
#pragma unroll
  for (int i = 0; i < B; ++i)
#pragma unroll
    for (int j = 0; j < B; ++j) o[i * B + j] = inv[i][j];
  // the fp32 copy of the mixed-precision solve, without a conversion pass
  if (dinv32) {
    float* o32 = dinv32 + static_cast<int64_t>(r) * B * B;
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
      for (int j = 0; j < B; ++j) o32[i * B + j] = static_cast<float>(inv[i][j]);
  }
}

template <int B, class V, class X>
__global__ void k_bj_apply(int nrows, const V* dinv, const X* x, X* y) {
  const int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (row >= static_cast<int64_t>(nrows) * B) return;
  const int br = static_cast<int>(row / B), i = static_cast<int>(row % B);
  const V* d = dinv + static_cast<int64_t>(br) * B * B + i * B;
  const X* xb = x + static_cast<int64_t>(br) * B;
  V acc = V(0);
#pragma unroll
  for (int j = 0; j < B; ++j) acc += d[j] * static_cast<V>(xb[j]);
  y[row] = static_cast<X>(acc);
}

template <class V, class X>
void bj_apply_dispatch(int nrows, int bs, const V* dinv, const X* x, X* y, cudaStream_t s) {
  const int64_t n = static_cast<int64_t>(nrows) * bs;
  if (n == 0) return;
  const int threads = 256;
  const int blocks = static_cast<int>((n + threads - 1) / threads);
  count_launches(1);
#define DC_BJ(B) \
  case B: k_bj_apply<B, V, X><<<blocks, threads, 0, s>>>(nrows, dinv, x, y); return;
  switch (bs) {
    DC_BJ(1) DC_BJ(2) DC_BJ(3) DC_BJ(4) DC_BJ(5) DC_BJ(6) DC_BJ(7) DC_BJ(8)
    default: throw std::runtime_error("block Jacobi: block size unsupported");
  }
#undef DC_BJ
}

// ---------------------------------------------------------------- elementwise

inline int ew_blocks(int64_t n) {
  count_launches(1);  // every elementwise launch sizes its grid through here
  int64_t b = (n + 255) / 256;
  return static_cast<int>(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

__global__ void k_axpby(int64_t n, double a, const double* x, double b, double* y) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = a * x[i] + b * y[i];
}
__global__ void k_axpy(int64_t n, double a, const double* x, double* y) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] += a * x[i];
}
// out = a x + b y with x or y optional; the rounding is that of y1 = a x, then y1 += b y
__global__ void k_combine(int64_t n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                          double* __restrict__ out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double ax = x ? a * x[i] : 0.0;
    out[i] = y ? __fma_rn(b, y[i], ax) : ax;
  }
}
__global__ void k_scale_copy(int64_t n, double a, const double* x, double* y) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = a * x[i];
}
__global__ void k_to_float(int64_t n, const double* x, double sc, float* y) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = static_cast<float>(x[i] * sc);
}
__global__ void k_add_float(int64_t n, const float* x, double sc, double* y) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] += sc * static_cast<double>(x[i]);
}
__global__ void k_fill(int64_t n, double v, double* y) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = v;
}

}  // namespace

static std::atomic<long long> g_launches{0};
static thread_local long long t_launches = 0;
long long launch_count() { return g_launches.load(); }
long long launch_count_this_thread() { return t_launches; }
void count_launches(long long n) {
  g_launches.fetch_add(n, std::memory_order_relaxed);
  t_launches += n;
}

void spmv(const Bsr& A, const double* x, double* y, cudaStream_t s) {
  spmv_dispatch<double, double>(A, A.val, x, y, nullptr, s);
}
void spmv32(const Bsr& A, const float* x, float* y, cudaStream_t s) {
  spmv_dispatch<float, float>(A, A.val32, x, y, nullptr, s);
}

namespace {

// one thread per (slice, lane): copies the lane's blocks into its SELL slots as fp32 and
// zero-fills the slots past the end of its row; the 32 lanes of a slice write each slot
// entry as one contiguous 128-byte line
template <int B, class O>
__global__ void __launch_bounds__(256) k_bsr_to_sell(Sell S, const int32_t* __restrict__ rowptr,
                                                     const double* __restrict__ val, O* __restrict__ out) {
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= S.nslices * 32) return;
  const int64_t sl = t >> 5;
  const int lane = static_cast<int>(t & 31);
  const int64_t o0 = S.off[sl];
  const int w = static_cast<int>(S.off[sl + 1] - o0);
  int k0 = 0, len = 0;
  if (t < S.nrows) {
    k0 = rowptr[t];
    len = rowptr[t + 1] - k0;
  }
  for (int k = 0; k < w; ++k) {
    O* dst = out + (o0 + k) * 32 * (B * B) + lane;
    const double* src = val + static_cast<int64_t>(k0 + k) * (B * B);
#pragma unroll
    for (int e = 0; e < B * B; ++e) dst[e * 32] = k < len ? static_cast<O>(src[e]) : O(0);
  }
}

template <int B>
__global__ void __launch_bounds__(256) k_sell_spmv(Sell S, const float* __restrict__ val, const float* __restrict__ x,
                                                   float* __restrict__ y) {
  const int64_t sl = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (sl >= S.nslices) return;
  const int lane = threadIdx.x & 31;
  float acc[B];
  sell_lane_rows<B, float, float>(S, sl, lane, val, x, acc);
  const int64_t br = sl * 32 + lane;
  if (br < S.nrows)
#pragma unroll
    for (int i = 0; i < B; ++i) y[br * B + i] = acc[i];
}

}  // namespace

template <class O>
void bsr_to_sell_t(const Bsr& A, const double* val, const Sell& S, O* out, cudaStream_t s) {
  if (S.nslices == 0) return;
  const int threads = 256;
  const int blocks = static_cast<int>((S.nslices * 32 + threads - 1) / threads);
  count_launches(1);
#define DC_B2S(B) \
  case B: k_bsr_to_sell<B, O><<<blocks, threads, 0, s>>>(S, A.rowptr, val, out); return;
  switch (S.bs) {
    DC_B2S(1) DC_B2S(2) DC_B2S(3) DC_B2S(4) DC_B2S(5) DC_B2S(6) DC_B2S(7) DC_B2S(8)
    default: throw std::runtime_error("sell: block size unsupported");
  }
#undef DC_B2S
}

void bsr_to_sell(const Bsr& A, const double* val, const Sell& S, float* out, cudaStream_t s) {
  bsr_to_sell_t<float>(A, val, S, out, s);
}
void bsr_to_sell64(const Bsr& A, const double* val, const Sell& S, double* out, cudaStream_t s) {
  bsr_to_sell_t<double>(A, val, S, out, s);
}

void spmv_sell32(const Sell& S, const float* val, const float* x, float* y, cudaStream_t s) {
  if (S.nslices == 0) return;
  const int threads = 256;
  const int blocks = static_cast<int>((S.nslices * 32 + threads - 1) / threads);
  count_launches(1);
#define DC_SS(B) \
  case B: k_sell_spmv<B><<<blocks, threads, 0, s>>>(S, val, x, y); return;
  switch (S.bs) {
    DC_SS(1) DC_SS(2) DC_SS(3) DC_SS(4) DC_SS(5) DC_SS(6) DC_SS(7) DC_SS(8)
    default: throw std::runtime_error("sell: block size unsupported");
  }
#undef DC_SS
}

void spmv32_vals(const Bsr& A, const float* val, const float* x, float* y, cudaStream_t s) {
  spmv_dispatch<float, float>(A, val, x, y, nullptr, s);
}
void residual(const Bsr& A, const double* x, const double* b, double* r, cudaStream_t s) {
  spmv_dispatch<double, double>(A, A.val, x, r, b, s);
}
void spmv_acc(const Bsr& A, const double* vals, const double* x, double* y, double alpha, cudaStream_t s) {
  spmv_dispatch<double, double>(A, vals, x, y, nullptr, s, alpha, 1);
}

void dot(const double* x, const double* y, int64_t n, ReduceScratch rs, int slot, cudaStream_t s) {
  reduce<1>(n, DotBody{x, y}, StoreFin{rs.result + slot}, rs, s);
}

void block_jacobi_setup(const Bsr& A, const int32_t* diag, double* dinv, int* status, cudaStream_t s,
                        float* dinv32) {
  if (A.nrows == 0) return;
  const int threads = 128, blocks = (A.nrows + threads - 1) / threads;
  count_launches(1);
#define DC_BJS(B) \
  case B: k_bj_setup<B><<<blocks, threads, 0, s>>>(A.nrows, diag, A.val, dinv, status, dinv32); return;
  switch (A.bs) {
    DC_BJS(1) DC_BJS(2) DC_BJS(3) DC_BJS(4) DC_BJS(5) DC_BJS(6) DC_BJS(7) DC_BJS(8)
    default: throw std::runtime_error("block Jacobi: block size unsupported");
  }
#undef DC_BJS
}
void block_jacobi_apply(int nrows, int bs, const double* dinv, const double* x, double* y, cudaStream_t s) {
  bj_apply_dispatch<double, double>(nrows, bs, dinv, x, y, s);
}
void block_jacobi_apply32(int nrows, int bs, const float* dinv, const float* x, float* y, cudaStream_t s) {
  bj_apply_dispatch<float, float>(nrows, bs, dinv, x, y, s);
}

void axpy(int64_t n, double a, const double* x, double* y, cudaStream_t s) {
  if (n > 0) k_axpy<<<ew_blocks(n), 256, 0, s>>>(n, a, x, y);
}
void axpby(int64_t n, double a, const double* x, double b, double* y, cudaStream_t s) {
  if (n > 0) k_axpby<<<ew_blocks(n), 256, 0, s>>>(n, a, x, b, y);
}
void scale_copy(int64_t n, double a, const double* x, double* y, cudaStream_t s) {
  if (n > 0) k_scale_copy<<<ew_blocks(n), 256, 0, s>>>(n, a, x, y);
}
void combine(int64_t n, double a, const double* x, double b, const double* y, double* out, cudaStream_t s) {
  if (n > 0) k_combine<<<ew_blocks(n), 256, 0, s>>>(n, a, x, b, y, out);
}
namespace {
__global__ void k_scatter_idx(int64_t n, const int64_t* __restrict__ idx, const double* __restrict__ src,
                              double* __restrict__ dst) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) dst[idx[i]] = src[i];
}
__global__ void k_gather_idx(int64_t n, const int64_t* __restrict__ idx, const double* __restrict__ src,
                             double* __restrict__ dst) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}
}  // namespace

void scatter_idx(int64_t n, const int64_t* idx, const double* src, double* dst, cudaStream_t s) {
  if (n <= 0) return;
  count_launches(1);
  k_scatter_idx<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(n, idx, src, dst);
}
void gather_idx(int64_t n, const int64_t* idx, const double* src, double* dst, cudaStream_t s) {
  if (n <= 0) return;
  count_launches(1);
  k_gather_idx<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(n, idx, src, dst);
}

void to_float(int64_t n, const double* x, float* y, cudaStream_t s) {
  if (n > 0) k_to_float<<<ew_blocks(n), 256, 0, s>>>(n, x, 1.0, y);
}
void to_float_scaled(int64_t n, const double* x, double scale, float* y, cudaStream_t s) {
  if (n > 0) k_to_float<<<ew_blocks(n), 256, 0, s>>>(n, x, scale, y);
}
void add_float(int64_t n, const float* x, double* y, cudaStream_t s) {
  if (n > 0) k_add_float<<<ew_blocks(n), 256, 0, s>>>(n, x, 1.0, y);
}
void add_float_scaled(int64_t n, const float* x, double scale, double* y, cudaStream_t s) {
  if (n > 0) k_add_float<<<ew_blocks(n), 256, 0, s>>>(n, x, scale, y);
}
void fill(int64_t n, double v, double* y, cudaStream_t s) {
  if (n > 0) k_fill<<<ew_blocks(n), 256, 0, s>>>(n, v, y);
}

}  // namespace dcgpu
