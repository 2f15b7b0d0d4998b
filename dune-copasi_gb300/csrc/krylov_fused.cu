// Single-launch preconditioned BiCGSTAB: the whole solve in one cooperative kernel.
//
// Replaces the same dune-istl BiCGSTABSolver as the five-kernel iteration in krylov.cu
// (dune/copasi/model/make_step_operator.hh:102-146, solver/istl/factory/iterative.hh:76-109).
// On problems whose operator and vectors sit in L2, an iteration's time is set by latency:
// each phase ends in a wait for the slowest block, and each SpMV's dependent loads.  Here
// the phases are separated by grid-wide barriers of a cooperative launch (about 2 us each
// at 304 blocks on GB300) instead of kernel boundaries, the SELL variant runs three phases
// instead of five, and the convergence test runs on the device, so a whole solve costs one
// launch and one read of the device scalars.
#include "krylov.cuh"

#include <algorithm>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace dcgpu {

namespace {

constexpr int kFThreads = 512;
constexpr int kFWarps = kFThreads / 32;
constexpr int kFMinBlocksPerSm = 2;
// Largest block size for which the three-phase iteration (each SpMV forming the
// preconditioned vector per gathered column) is used.  It trades two phases and their
// barriers for 3B + B^2 values gathered per column instead of B: a gain while the operator
// sits in L2 and the iteration is latency-bound (Gray-Scott 512^2, B = 2: 43 -> 38 us per
// iteration), a loss once the gathers compete for HBM bandwidth (3D cross-diffusion 128^3,
// B = 3: 55 % of the HBM peak against 73 % with five phases).
constexpr int kThreePhaseMaxB = 2;
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier over the co-resident blocks of a cooperative launch.  bar[0] counts
// arrivals, bar[1] holds the generation.  The last block to arrive resets the counter and
// publishes the next generation; the others poll it, for at most kBarrierTimeoutNs.
// Returns false in every thread of the block when the wait gave up.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned& gen,
                                             unsigned long long timeout_ns = kBarrierTimeoutNs) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int good = 1;
    const unsigned next = gen + 1u;
    __threadfence();
    if (atomicAdd(&bar[0], 1u) == gridDim.x - 1) {
      atomicExch(&bar[0], 0u);
      __threadfence();
      atomicExch(&bar[1], next);
    } else {
      const unsigned long long t0 = global_ns();
      while (*reinterpret_cast<volatile unsigned*>(&bar[1]) != next) {
        if (global_ns() - t0 > timeout_ns) {
          good = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    gen = next;
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Block sums of the threads' partial sums acc, stored by thread 0 at part[blockIdx.x * N +
// k].  A thread accumulates its few elements, and a warp its 32 threads, in the vector
// precision A; the sums across warps and blocks are FP64.  (GB300's FP64 rate is 1/58 of
// its FP32 rate: per-element FP64 products and conversions, and FP64 shuffles in every
// warp, made the fp32 solve's reductions FP64-bound.)
template <int N, class A>
__device__ __forceinline__ void block_partials(const A (&acc)[N], double* part) {
  __shared__ double sh[N][kFWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    A v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][warp] = static_cast<double>(v);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double v = 0.0;
      for (int w = 0; w < kFWarps; ++w) v += sh[k][w];
      __stcg(part + static_cast<int64_t>(blockIdx.x) * N + k, v);
    }
  }
}

// Sums over all blocks of the stored partials, in block order, left in thread 0 (warp 0
// reads and adds them; every block computes the same bits).
template <int N>
__device__ __forceinline__ void grid_totals0(const double* part, double (&out)[N]) {
  if (threadIdx.x >= 32) return;
  double acc[N];
#pragma unroll
  for (int k = 0; k < N; ++k) acc[k] = 0.0;
  // a lane's partials (blocks lane, lane + 32, ...) are loaded 8 at a time before they are
  // added, so their L2 latencies overlap
  constexpr int U = 8;
  const int G = static_cast<int>(gridDim.x);
  for (int b0 = 0; b0 < G; b0 += 32 * U) {
    double v[U][N];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int b = b0 + u * 32 + static_cast<int>(threadIdx.x);
#pragma unroll
      for (int k = 0; k < N; ++k) v[u][k] = b < G ? __ldcg(part + static_cast<int64_t>(b) * N + k) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < N; ++k) acc[k] += v[u][k];
  }
#pragma unroll
  for (int k = 0; k < N; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    out[k] = acc[k];
  }
}

// The BiCGSTAB scalars, kept in shared memory: thread 0 of every block updates them from
// the grid totals (all blocks hold the same bits, so they take the same decisions) and the
// other threads read them after a block barrier.
struct BicgScalars {
  double rho, rho_new, alpha, omega, beta, rv, ts, tt, rr, rr0, target, done;
  int it;
};

__device__ __forceinline__ void scalars_init(BicgScalars& S, double rr, double rel) {
  S.rr = S.rr0 = S.rho = S.rho_new = rr;
  S.target = rel * rel * rr;
  S.alpha = S.omega = S.beta = 1.0;
  S.rv = S.ts = S.tt = 0.0;
  S.done = !isfinite(rr) ? kDoneNonFinite : (rr == 0.0 ? kDoneConverged : 0.0);
  S.it = 0;
}

// alpha = rho / <rhat, v>
__device__ __forceinline__ void scalars_rv(BicgScalars& S, double rv) {
  S.rv = rv;
  const double q = S.rho / rv;
  if (!isfinite(rv)) S.done = kDoneNonFinite;
  else if (rv == 0.0 || !isfinite(q)) S.done = kDoneBreakdown;
  S.alpha = isfinite(q) ? q : 0.0;
}

// omega = <t, s> / <t, t>
__device__ __forceinline__ void scalars_omega(BicgScalars& S, double ts, double tt) {
  S.ts = ts;
  S.tt = tt;
  double w = tt != 0.0 ? ts / tt : 0.0;
  if (!isfinite(w)) {
    S.done = kDoneNonFinite;
    w = 0.0;
  }
  S.omega = w;
}

// ||r||^2, <rhat, r>: convergence test, beta, rho
__device__ __forceinline__ void scalars_rr(BicgScalars& S, double rr, double rho_new) {
  S.rr = rr;
  S.rho_new = rho_new;
  S.it += 1;
  if (!isfinite(rr) || !isfinite(rho_new)) {
    S.done = kDoneNonFinite;
    return;
  }
  if (rr <= S.target) {
    S.done = kDoneConverged;
    return;
  }
  const double bt = (rho_new / S.rho) * (S.alpha / S.omega);
  if (rho_new == 0.0 || S.omega == 0.0 || !isfinite(bt)) {
    S.done = kDoneBreakdown;
    return;
  }
  S.beta = bt;
  S.rho = rho_new;
}

__device__ __forceinline__ void scalars_store(const BicgScalars& S, double* sc) {
  sc[KS_RR] = S.rr;
  sc[KS_RR0] = S.rr0;
  sc[KS_TARGET] = S.target;
  sc[KS_RHO] = S.rho;
  sc[KS_RHONEW] = S.rho_new;
  sc[KS_ALPHA] = S.alpha;
  sc[KS_OMEGA] = S.omega;
  sc[KS_BETA] = S.beta;
  sc[KS_RV] = S.rv;
  sc[KS_TS] = S.ts;
  sc[KS_TT] = S.tt;
  sc[KS_ITER] = static_cast<double>(S.it);
  sc[KS_DONE] = S.done;
}

// y = A x with acc[0] += <w, y> and, for N == 2, acc[1] += <y, y>; x is read through L2
template <int B, class T, class V, bool SELL, int N>
__device__ __forceinline__ void spmv_dots(const FusedBicgArgs<T, V>& a, const T* __restrict__ x, T* __restrict__ y,
                                          const T* __restrict__ w, T (&acc)[N], int gtid, int gstride) {
  if constexpr (SELL) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = gstride >> 5;
    for (int64_t sl = gtid >> 5; sl < a.S.nslices; sl += nw) {
      V yv[B];
      sell_lane_rows<B, T, V, true>(a.S, sl, lane, a.vals, x, yv);
      const int64_t br = sl * 32 + lane;
      if (br < a.nrows) {
#pragma unroll
        for (int i = 0; i < B; ++i) {
          const T yt = static_cast<T>(yv[i]);
          y[br * B + i] = yt;
          acc[0] += __ldcg(w + br * B + i) * yt;
          if constexpr (N == 2) acc[1] += yt * yt;
        }
      }
    }
  } else {
    const int64_t n = static_cast<int64_t>(a.nrows) * B;
    for (int64_t row = gtid; row < n; row += gstride) {
      const int br = static_cast<int>(row / B), i = static_cast<int>(row % B);
      V yv = V(0);
      const int k0 = __ldg(a.rowptr + br), k1 = __ldg(a.rowptr + br + 1);
      for (int k = k0; k < k1; ++k) {
        const int c = __ldg(a.colidx + k);
        const V* blk = a.vals + static_cast<int64_t>(k) * B * B + i * B;
        const T* xc = x + static_cast<int64_t>(c) * B;
#pragma unroll
        for (int j = 0; j < B; ++j) yv += __ldg(blk + j) * static_cast<V>(__ldcg(xc + j));
      }
      const T yt = static_cast<T>(yv);
      y[row] = yt;
      acc[0] += __ldcg(w + row) * yt;
      if constexpr (N == 2) acc[1] += yt * yt;
    }
  }
}

// hat = D^-1 in for block row nd (block-Jacobi apply)
template <int B, class T, class V>
__device__ __forceinline__ void jacobi_row(const V* __restrict__ dinv, int nd, const V (&in)[B], T* __restrict__ hat) {
  const V* d = dinv + static_cast<int64_t>(nd) * B * B;
  const int64_t o = static_cast<int64_t>(nd) * B;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    V acc = V(0);
#pragma unroll
    for (int j = 0; j < B; ++j) acc += __ldg(d + i * B + j) * in[j];
    hat[o + i] = static_cast<T>(acc);
  }
}

// The vector the SpMV multiplies, formed for block row c from vectors of the previous
// phase: PU: u = r + c1 (p - c2 v) (the p update, c1 = beta, c2 = omega); otherwise
// u = r - c1 v (the s update, c1 = alpha).  Same V arithmetic as the stored p / s.
template <int B, class T, class V, bool PU>
__device__ __forceinline__ void combine_row(int64_t c, const T* __restrict__ r, const T* __restrict__ p,
                                            const T* __restrict__ v, V c1, V c2, V (&u)[B]) {
  T rv[B], vv[B];
  load_block<B, true>(r + c * B, rv);
  load_block<B, true>(v + c * B, vv);
  if constexpr (PU) {
    T pv[B];
    load_block<B, true>(p + c * B, pv);
#pragma unroll
    for (int j = 0; j < B; ++j)
      u[j] = static_cast<V>(rv[j]) + c1 * (static_cast<V>(pv[j]) - c2 * static_cast<V>(vv[j]));
  } else {
#pragma unroll
    for (int j = 0; j < B; ++j) u[j] = static_cast<V>(rv[j]) - c1 * static_cast<V>(vv[j]);
  }
}

// D_c^-1 u rounded to T, as the stored preconditioned vector would hold it
template <int B, class T, class V>
__device__ __forceinline__ void jacobi_apply(const V* __restrict__ dinv, int64_t c, const V (&u)[B], V (&out)[B]) {
  V d[B * B];
  load_block<B * B, false>(dinv + c * B * B, d);
#pragma unroll
  for (int i = 0; i < B; ++i) {
    V acc = V(0);
#pragma unroll
    for (int j = 0; j < B; ++j) acc += d[i * B + j] * u[j];
    out[i] = static_cast<V>(static_cast<T>(acc));
  }
}

// y rows of SELL slice sl for lane `lane` with the multiplied vector formed per gathered
// column: y = A (D^-1 u), u from combine_row.  Slots in batches of two, as in
// sell_lane_rows, so that the gathers of two columns are in flight together.
template <int B, class T, class V, bool PU>
__device__ __forceinline__ void sell_rows_jacobi(const Sell& S, int64_t sl, int lane, const V* __restrict__ val,
                                                 const V* __restrict__ dinv, const T* __restrict__ r,
                                                 const T* __restrict__ p, const T* __restrict__ v, V c1, V c2,
                                                 V (&acc)[B]) {
#pragma unroll
  for (int i = 0; i < B; ++i) acc[i] = V(0);
  const int64_t o0 = S.off[sl], o1 = S.off[sl + 1];
  const int32_t* __restrict__ cols = S.cols + o0 * 32 + lane;
  const V* __restrict__ vbase = val + o0 * 32 * (B * B) + lane;
  const int w = static_cast<int>(o1 - o0);
  constexpr int U = 2;
  // the column indices of the next batch are loaded while the current batch's gathers are
  // in flight, so a batch costs one L2 round trip, not two
  int cn[U];
#pragma unroll
  for (int q = 0; q < U; ++q) cn[q] = q < w ? __ldg(cols + q * 32) : 0;
  int k = 0;
  for (; k + U <= w; k += U) {
    int c[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      c[q] = cn[q];
      const int kn = k + U + q;
      cn[q] = kn < w ? __ldg(cols + kn * 32) : 0;
    }
    V u[U][B], xh[U][B];
#pragma unroll
    for (int q = 0; q < U; ++q) combine_row<B, T, V, PU>(c[q], r, p, v, c1, c2, u[q]);
#pragma unroll
    for (int q = 0; q < U; ++q) jacobi_apply<B, T, V>(dinv, c[q], u[q], xh[q]);
#pragma unroll
    for (int q = 0; q < U; ++q) {
      V blk[B * B];
      load_block_interleaved<B * B>(vbase + static_cast<int64_t>(k + q) * (32 * B * B), blk);
#pragma unroll
      for (int i = 0; i < B; ++i)
#pragma unroll
        for (int j = 0; j < B; ++j) acc[i] += blk[i * B + j] * xh[q][j];
    }
  }
  // the last w % U slots, whose columns are already in cn
#pragma unroll
  for (int q = 0; q < U - 1; ++q) {
    if (k + q >= w) break;
    const int c = cn[q];
    V u[B], xh[B];
    combine_row<B, T, V, PU>(c, r, p, v, c1, c2, u);
    jacobi_apply<B, T, V>(dinv, c, u, xh);
    V blk[B * B];
    load_block_interleaved<B * B>(vbase + static_cast<int64_t>(k + q) * (32 * B * B), blk);
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
      for (int j = 0; j < B; ++j) acc[i] += blk[i * B + j] * xh[j];
  }
}

// A grid-wide barrier whose wait gave up: flag it; the caller's whole block returns.
__device__ __forceinline__ bool barrier_or_fault(unsigned* bar, unsigned& gen, double* sc) {
  if (grid_barrier(bar, gen)) return true;
  if (threadIdx.x == 0) sc[KS_FAULT] = 1.0;
  return false;
}

// One BiCGSTAB solve of A x = r to the relative reduction rel in at most max_it iterations.
// With r64 set, r is first formed as r64 * scale (rounded to T), else read as it is.
// THREE (SELL-32 operator, block size <= kThreePhaseMaxB): three phases per iteration, the preconditioned
// vectors formed inside the SpMVs, p and v alternating between two buffers by iteration
// parity (p[cur], v[cur] written, p[prv], v[prv] read).  Otherwise five phases: p update
// with the Jacobi apply, SpMV, s update with the Jacobi apply, SpMV, x / r update.
// Returns false when a barrier wait gave up.
template <int B, class T, class V, bool SELL, bool THREE>
__device__ __forceinline__ bool bicg_solve(const FusedBicgArgs<T, V>& a, BicgScalars& S, unsigned* bar, unsigned& gen,
                                           const double* r64, double scale, double rel, int max_it) {
  const int G = static_cast<int>(gridDim.x);
  double* part_rv = a.partial;
  double* part_ts = a.partial + G;
  double* part_rr = a.partial + 3 * static_cast<int64_t>(G);
  const int gtid = blockIdx.x * kFThreads + threadIdx.x;
  const int gstride = G * kFThreads;
  const int lane = threadIdx.x & 31;
  const int64_t nw = gstride >> 5;
  const int nrows = a.nrows;
  const int64_t n = static_cast<int64_t>(nrows) * B;

  // x = 0, rhat = r, the p and v read by iteration 0 = 0, ||r||^2
  {
    T a1[1] = {T(0)};
    T* p0 = THREE ? a.p2 : a.p;
    T* v0 = THREE ? a.v2 : a.v;
    for (int64_t i = gtid; i < n; i += gstride) {
      T ri;
      if (r64) {
        ri = static_cast<T>(__ldcg(r64 + i) * scale);
        a.r[i] = ri;
      } else {
        ri = __ldcg(a.r + i);
      }
      a.rhat[i] = ri;
      p0[i] = T(0);
      v0[i] = T(0);
      a.x[i] = T(0);
      a1[0] += ri * ri;
    }
    block_partials<1>(a1, part_rv);
  }
  if (!barrier_or_fault(bar, gen, a.sc)) return false;
  {
    double t1[1];
    grid_totals0<1>(part_rv, t1);
    if (threadIdx.x == 0) scalars_init(S, t1[0], rel);
  }
  __syncthreads();

  for (;;) {
    if (S.done != 0.0 || S.it >= max_it) break;
    const int cur = S.it & 1;
    const V bv = static_cast<V>(S.beta), ov = static_cast<V>(S.omega);
    T* pc = (THREE && cur) ? a.p2 : a.p;
    T* vc = (THREE && cur) ? a.v2 : a.v;
    const T* pp = (THREE && !cur) ? a.p2 : a.p;
    const T* vp = (THREE && !cur) ? a.v2 : a.v;

    // (1) v = A phat, phat = D^-1 (r + beta (p - omega v));  <rhat, v>
    if constexpr (THREE) {
      T acc[1] = {T(0)};
      for (int64_t sl = gtid >> 5; sl < a.S.nslices; sl += nw) {
        V y[B];
        sell_rows_jacobi<B, T, V, true>(a.S, sl, lane, a.vals, a.dinv, a.r, pp, vp, bv, ov, y);
        const int64_t br = sl * 32 + lane;
        if (br < nrows) {
          V u[B];
          combine_row<B, T, V, true>(br, a.r, pp, vp, bv, ov, u);
#pragma unroll
          for (int i = 0; i < B; ++i) pc[br * B + i] = static_cast<T>(u[i]);
          jacobi_row<B, T, V>(a.dinv, static_cast<int>(br), u, a.phat);
#pragma unroll
          for (int i = 0; i < B; ++i) {
            const T yt = static_cast<T>(y[i]);
            vc[br * B + i] = yt;
            acc[0] += __ldcg(a.rhat + br * B + i) * yt;
          }
        }
      }
      block_partials<1>(acc, part_rv);
    } else {
      for (int nd = gtid; nd < nrows; nd += gstride) {
        V u[B];
        combine_row<B, T, V, true>(nd, a.r, a.p, a.v, bv, ov, u);
#pragma unroll
        for (int i = 0; i < B; ++i) a.p[static_cast<int64_t>(nd) * B + i] = static_cast<T>(u[i]);
        jacobi_row<B, T, V>(a.dinv, nd, u, a.phat);
      }
      if (!barrier_or_fault(bar, gen, a.sc)) return false;
      T acc[1] = {T(0)};
      spmv_dots<B, T, V, SELL, 1>(a, a.phat, a.v, a.rhat, acc, gtid, gstride);
      block_partials<1>(acc, part_rv);
    }
    if (!barrier_or_fault(bar, gen, a.sc)) return false;
    {
      double t1[1];
      grid_totals0<1>(part_rv, t1);
      if (threadIdx.x == 0) scalars_rv(S, t1[0]);
    }
    __syncthreads();
    if (S.done != 0.0) break;
    const V av = static_cast<V>(S.alpha);

    // (2) t = A shat, shat = D^-1 (r - alpha v);  <t, s>, <t, t>
    if constexpr (THREE) {
      T acc[2] = {T(0), T(0)};
      for (int64_t sl = gtid >> 5; sl < a.S.nslices; sl += nw) {
        V y[B];
        sell_rows_jacobi<B, T, V, false>(a.S, sl, lane, a.vals, a.dinv, a.r, nullptr, vc, av, V(0), y);
        const int64_t br = sl * 32 + lane;
        if (br < nrows) {
          V u[B];
          combine_row<B, T, V, false>(br, a.r, nullptr, vc, av, V(0), u);
          T st[B];
#pragma unroll
          for (int i = 0; i < B; ++i) {
            st[i] = static_cast<T>(u[i]);
            a.s[br * B + i] = st[i];
          }
          jacobi_row<B, T, V>(a.dinv, static_cast<int>(br), u, a.shat);
#pragma unroll
          for (int i = 0; i < B; ++i) {
            const T yt = static_cast<T>(y[i]);
            a.t[br * B + i] = yt;
            acc[0] += yt * st[i];
            acc[1] += yt * yt;
          }
        }
      }
      block_partials<2>(acc, part_ts);
    } else {
      for (int nd = gtid; nd < nrows; nd += gstride) {
        V u[B];
        combine_row<B, T, V, false>(nd, a.r, nullptr, a.v, av, V(0), u);
#pragma unroll
        for (int i = 0; i < B; ++i) a.s[static_cast<int64_t>(nd) * B + i] = static_cast<T>(u[i]);
        jacobi_row<B, T, V>(a.dinv, nd, u, a.shat);
      }
      if (!barrier_or_fault(bar, gen, a.sc)) return false;
      T acc[2] = {T(0), T(0)};
      spmv_dots<B, T, V, SELL, 2>(a, a.shat, a.t, a.s, acc, gtid, gstride);
      block_partials<2>(acc, part_ts);
    }
    if (!barrier_or_fault(bar, gen, a.sc)) return false;
    {
      double t2[2];
      grid_totals0<2>(part_ts, t2);
      if (threadIdx.x == 0) scalars_omega(S, t2[0], t2[1]);
    }
    __syncthreads();
    if (S.done != 0.0) break;

    // (3) x += alpha phat + omega shat;  r = s - omega t;  ||r||^2, <rhat, r>
    {
      const T al = static_cast<T>(S.alpha), om = static_cast<T>(S.omega);
      T acc[2] = {T(0), T(0)};
      for (int64_t i = gtid; i < n; i += gstride) {
        a.x[i] = __ldcg(a.x + i) + al * __ldcg(a.phat + i) + om * __ldcg(a.shat + i);
        const T ri = __ldcg(a.s + i) - om * __ldcg(a.t + i);
        a.r[i] = ri;
        acc[0] += ri * ri;
        acc[1] += __ldcg(a.rhat + i) * ri;
      }
      block_partials<2>(acc, part_rr);
    }
    if (!barrier_or_fault(bar, gen, a.sc)) return false;
    {
      double t2[2];
      grid_totals0<2>(part_rr, t2);
      if (threadIdx.x == 0) scalars_rr(S, t2[0], t2[1]);
    }
    __syncthreads();
  }
  return true;
}

// fp64 residual r64 = b64 - J z64 (one thread per scalar row, as the fp64 BSR SpMV) and
// its squared norm into the block partials
template <int B, class T, class V>
__device__ __forceinline__ void residual64(const FusedBicgArgs<T, V>& a, double* part) {
  const int gtid = blockIdx.x * kFThreads + threadIdx.x;
  const int gstride = static_cast<int>(gridDim.x) * kFThreads;
  const int64_t n = static_cast<int64_t>(a.nrows) * B;
  double acc[1] = {0.0};
  for (int64_t row = gtid; row < n; row += gstride) {
    const int br = static_cast<int>(row / B), i = static_cast<int>(row % B);
    double y = 0.0;
    const int k0 = __ldg(a.rowptr + br), k1 = __ldg(a.rowptr + br + 1);
    for (int k = k0; k < k1; ++k) {
      const int c = __ldg(a.colidx + k);
      const double* blk = a.vals64 + static_cast<int64_t>(k) * B * B + i * B;
      const double* zc = a.z64 + static_cast<int64_t>(c) * B;
#pragma unroll
      for (int j = 0; j < B; ++j) y += __ldg(blk + j) * __ldcg(zc + j);
    }
    const double r = __ldg(a.b64 + row) - y;
    a.r64[row] = r;
    acc[0] += r * r;
  }
  block_partials<1>(acc, part);
}

// the refinement's state, kept in shared memory like the BiCGSTAB scalars
struct RefineState {
  double rn, target;
  int total, refs, status;   // status: 0 running, 1 converged, 2 diverged, 3 out of iterations
};

template <int B, class T, class V, bool SELL, bool THREE>
__global__ void __launch_bounds__(kFThreads, kFMinBlocksPerSm) k_bicgstab_single(FusedBicgArgs<T, V> a) {
  static_assert(SELL || !THREE, "the three-phase iteration runs on the SELL operator");
  __shared__ BicgScalars S;
  __shared__ RefineState R;
  unsigned* bar = reinterpret_cast<unsigned*>(a.sc + KS_BARRIER);
  unsigned gen = 0;
  if (!a.b64) {
    if (!bicg_solve<B, T, V, SELL, THREE>(a, S, bar, gen, nullptr, 1.0, a.rel, a.max_it)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) scalars_store(S, a.sc);
    return;
  }

  // refined solve: z = 0, |b|
  const int gtid = blockIdx.x * kFThreads + threadIdx.x;
  const int gstride = static_cast<int>(gridDim.x) * kFThreads;
  const int64_t n = static_cast<int64_t>(a.nrows) * B;
  double* part = a.partial + 3 * static_cast<int64_t>(gridDim.x);   // the ||r||^2 partials
  {
    double acc[1] = {0.0};
    for (int64_t i = gtid; i < n; i += gstride) {
      a.z64[i] = 0.0;
      const double bi = __ldg(a.b64 + i);
      acc[0] += bi * bi;
    }
    block_partials<1>(acc, part);
  }
  if (!barrier_or_fault(bar, gen, a.sc)) return;
  {
    double t1[1];
    grid_totals0<1>(part, t1);
    if (threadIdx.x == 0) {
      const double b0 = sqrt(t1[0]);
      R.rn = b0;
      R.target = a.rel * b0;
      R.total = 0;
      R.refs = 0;
      R.status = b0 == 0.0 ? 1 : (!isfinite(b0) ? 2 : 0);
    }
  }
  __syncthreads();

  for (int ref = 0; R.status == 0 && ref < a.max_refinements && R.total < a.max_it; ++ref) {
    if (ref > 0) {
      // r = b - J z and its norm decide whether another correction is needed
      residual64<B, T, V>(a, part);
      if (!barrier_or_fault(bar, gen, a.sc)) return;
      double t1[1];
      grid_totals0<1>(part, t1);
      if (threadIdx.x == 0) {
        R.rn = sqrt(t1[0]);
        if (!isfinite(R.rn)) R.status = 2;
        else if (R.rn <= R.target) R.status = 1;
      }
      __syncthreads();
      if (R.status != 0) break;
    }
    // the correction equation J d = r / |r| in T, then z += |r| d
    const double rn = R.rn;
    const double inner = fmax(a.inner, 0.5 * R.target / rn);
    if (!bicg_solve<B, T, V, SELL, THREE>(a, S, bar, gen, ref == 0 ? a.b64 : a.r64, 1.0 / rn, inner,
                                          a.max_it - R.total))
      return;
    if (threadIdx.x == 0) {
      R.refs += 1;
      R.total += S.it;
      if (S.it == 0 && (S.done == kDoneBreakdown || S.done == kDoneNonFinite)) R.status = 2;
    }
    __syncthreads();
    if (R.status != 0) break;
    for (int64_t i = gtid; i < n; i += gstride) a.z64[i] += rn * static_cast<double>(__ldcg(a.x + i));
    if (!barrier_or_fault(bar, gen, a.sc)) return;
  }
  if (R.status == 0) {
    // out of corrections or iterations: the final residual decides
    residual64<B, T, V>(a, part);
    if (!barrier_or_fault(bar, gen, a.sc)) return;
    double t1[1];
    grid_totals0<1>(part, t1);
    if (threadIdx.x == 0) {
      R.rn = sqrt(t1[0]);
      R.status = R.rn <= R.target ? 1 : 3;
    }
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.sc[KS_ITER] = static_cast<double>(R.total);
    a.sc[KS_REFINEMENTS] = static_cast<double>(R.refs);
    a.sc[KS_RR] = R.rn * R.rn;
    a.sc[KS_DONE] = R.status == 1 ? kDoneConverged : (R.status == 2 ? kDoneBreakdown : 0.0);
  }
}

// Self-test of the bounded wait: one barrier whose arrival counter starts past the value
// its last arrival would reach, so it can never complete; every block must give up after
// timeout_ns, flag the fault and return.
__global__ void k_barrier_selftest(unsigned* bar, double* flag, unsigned long long timeout_ns) {
  unsigned gen = 0;
  if (!grid_barrier(bar, gen, timeout_ns) && threadIdx.x == 0) atomicAdd(flag, 1.0);
}

template <class T, class V>
const void* fused_kernel(int bs, bool sell) {
#define DC_FK(B)                                                                                   \
  case B:                                                                                          \
    if constexpr (std::is_same_v<V, float>) {                                                      \
      if constexpr (B <= kThreePhaseMaxB) {                                                        \
        if (sell) return reinterpret_cast<const void*>(&k_bicgstab_single<B, T, V, true, true>);   \
      }                                                                                            \
      if (sell) return reinterpret_cast<const void*>(&k_bicgstab_single<B, T, V, true, false>);    \
    }                                                                                              \
    return sell ? nullptr : reinterpret_cast<const void*>(&k_bicgstab_single<B, T, V, false, false>);
  switch (bs) {
    DC_FK(1) DC_FK(2) DC_FK(3) DC_FK(4) DC_FK(5) DC_FK(6) DC_FK(7) DC_FK(8)
    default: return nullptr;
  }
#undef DC_FK
}

}  // namespace

template <class T, class V>
bool fused_bicgstab_plan(int bs, bool sell, int nrows, int* blocks, int* slots, int* capacity) {
  const void* k = fused_kernel<T, V>(bs, sell);
  if (!k || nrows <= 0) return false;
  int dev = 0, coop = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kFThreads, 0) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (!coop || per_sm < 1) return false;
  // a block of a kernel that fits per_sm (< kFMinBlocksPerSm) blocks on an SM holds
  // kFMinBlocksPerSm / per_sm slots of it
  const int per = std::min(per_sm, kFMinBlocksPerSm);
  const int64_t cap = static_cast<int64_t>(sms) * per;
  // one thread per scalar row (BSR SpMV) or per block row (vector phases, SELL lanes)
  const int64_t rows = sell ? nrows : static_cast<int64_t>(nrows) * bs;
  const int64_t need = (rows + kFThreads - 1) / kFThreads;
  *blocks = static_cast<int>(std::max<int64_t>(1, std::min(need, cap)));
  *slots = *blocks * (kFMinBlocksPerSm / per);
  *capacity = sms * kFMinBlocksPerSm;
  return true;
}

template <class T, class V>
void fused_bicgstab(int bs, bool sell, int blocks, const FusedBicgArgs<T, V>& a, cudaStream_t s) {
  const void* k = fused_kernel<T, V>(bs, sell);
  if (!k) throw std::runtime_error("fused BiCGSTAB: block size " + std::to_string(bs) + " unsupported");
  if (cudaMemsetAsync(a.sc + KS_FAULT, 0, 2 * sizeof(double), s) != cudaSuccess)
    throw std::runtime_error("fused BiCGSTAB: memset failed");
  FusedBicgArgs<T, V> copy = a;
  void* args[] = {&copy};
  const cudaError_t e = cudaLaunchCooperativeKernel(k, dim3(blocks), dim3(kFThreads), args, 0, s);
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("fused BiCGSTAB launch failed: ") + cudaGetErrorString(e));
  count_launches(1);
}

int barrier_selftest(double* gave_up_blocks, double* elapsed_ms) {
  constexpr int kBlocks = 4;
  constexpr unsigned long long kTimeoutNs = 50000000ull;  // 50 ms
  unsigned* bar = nullptr;
  double* flag = nullptr;
  if (cudaMalloc(&bar, 2 * sizeof(unsigned)) != cudaSuccess) return 1;
  if (cudaMalloc(&flag, sizeof(double)) != cudaSuccess) {
    cudaFree(bar);
    return 1;
  }
  // counter far past kBlocks - 1: no arrival ever sees the last-arrival value
  const unsigned init[2] = {1000u, 0u};
  cudaMemcpy(bar, init, sizeof init, cudaMemcpyHostToDevice);
  cudaMemset(flag, 0, sizeof(double));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  unsigned long long t = kTimeoutNs;
  void* args[] = {&bar, &flag, &t};
  cudaEventRecord(a);
  cudaError_t e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(&k_barrier_selftest), dim3(kBlocks),
                                              dim3(32), args, 0, nullptr);
  cudaEventRecord(b);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float ms = 0.0f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
  double h = 0.0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, flag, sizeof(double), cudaMemcpyDeviceToHost);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(bar);
  cudaFree(flag);
  if (e != cudaSuccess) return 1;
  count_launches(1);
  *gave_up_blocks = h;
  *elapsed_ms = ms;
  return 0;
}

template bool fused_bicgstab_plan<float, float>(int, bool, int, int*, int*, int*);
template bool fused_bicgstab_plan<double, double>(int, bool, int, int*, int*, int*);
template void fused_bicgstab<float, float>(int, bool, int, const FusedBicgArgs<float, float>&, cudaStream_t);
template void fused_bicgstab<double, double>(int, bool, int, const FusedBicgArgs<double, double>&, cudaStream_t);

}  // namespace dcgpu
