// Continuous batching of block-Jacobi BiCGSTAB solves across simulations (batch.hpp).
//
// Per iteration the same five phases as the per-model solve (krylov.cu, the dune-istl
// BiCGSTABSolver recurrences the reference's LinearSolver drives,
// dune/copasi/model/make_step_operator.hh:102-146): (1) p = r + beta (p - omega v),
// phat = D^-1 p; (2) v = A phat, <rhat, v>, alpha; (3) s = r - alpha v, shat = D^-1 s;
// (4) t = A shat, <t, s>, <t, t>, omega; (5) x += alpha phat + omega shat, r = s - omega t,
// ||r||^2, <rhat, r>, beta and the convergence test.  Each phase is one kernel over the
// tile table of all instances in the batch: a block takes a tile (256 block rows of one
// instance; thread k owns block row k of the tile, warp w the SELL-32 slice w) and moves on
// to tile + gridDim.x.  Instances that converged skip their tiles.
#include "batch.hpp"

#include <algorithm>
#include <array>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "krylov.cuh"
#include "linalg.cuh"
#include "model.hpp"

namespace dcgpu {

namespace {

constexpr int kTileRows = 256;  // block rows per tile = threads per block
constexpr int kTileWarps = kTileRows / 32;
// BiCGSTAB iterations of the captured replays: a replay runs the shortest that covers the
// iterations the instance closest to convergence is expected to need
constexpr int kChunks[] = {2, 4, 8};
constexpr int kNumChunks = 3;
constexpr int kPhases = 5;      // kernels per iteration
constexpr double kDoneMaxIt = 4.0;  // KS_DONE: max_it iterations ran without convergence

template <class T>
struct BInst {
  int nrows, bs, first_tile, ntiles;
  double rel;
  int max_it, pad;
  Sell S;
  const T* vals;
  const T* dinv;
  T *x, *r, *rhat, *p, *v, *s, *t, *phat, *shat;
};

// Device-resident header of a lane (one precision); the captured kernels take its address,
// so a new batch composition is an upload, not a new graph.
template <class T>
struct BLane {
  int ntiles, ninit;
  const int2* tiles;       // (slot, tile of the instance) of every active instance
  const int2* init_tiles;  // the tiles of the instances admitted for this replay
  const BInst<T>* inst;    // per slot
  double* sc;              // per slot: KS_COUNT scalars
  double* part;            // two partial sums per tile, at (first_tile + tile) * 2
  unsigned int* cnt;       // per slot: tiles of the running phase that have finished
};

// Partial sums of one tile: per warp in the vector type A (one conversion per warp), the
// warps in order in fp64, stored at ipart[tile * 2 + k].  The block that stores the last
// tile of the instance in this phase adds the instance's tile partials in tile order (warp
// 0: lane-strided sums, then a fixed shuffle tree), resets the counter and returns true in
// thread 0 with the totals in tot.  The order of every addition depends on the instance
// alone, never on which block ran which tile or on the other instances.
template <int NS, class A>
__device__ __forceinline__ bool tile_sum(const A (&part)[NS], double (&tot)[NS], double* ipart, int tile, int ntiles,
                                         unsigned int* cnt) {
  __shared__ double sh[NS][kTileWarps];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    A v = part[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][warp] = static_cast<double>(v);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      double v = 0.0;
      for (int w = 0; w < kTileWarps; ++w) v += sh[k][w];
      ipart[tile * 2 + k] = v;
    }
    __threadfence();
    last = atomicAdd(cnt, 1u) == static_cast<unsigned int>(ntiles - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NS; ++k) tot[k] = 0.0;
    for (int b = lane; b < ntiles; b += 32)
#pragma unroll
      for (int k = 0; k < NS; ++k) tot[k] += __ldcg(&ipart[b * 2 + k]);
#pragma unroll
    for (int k = 0; k < NS; ++k)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tot[k] += __shfl_down_sync(0xffffffffu, tot[k], o);
  }
  if (threadIdx.x == 0) *cnt = 0u;
  return threadIdx.x == 0;
}

#define DC_BT_DISPATCH(bs, CALL)       \
  switch (bs) {                        \
    case 1: CALL(1); break;            \
    case 2: CALL(2); break;            \
    case 3: CALL(3); break;            \
    case 4: CALL(4); break;            \
    case 5: CALL(5); break;            \
    case 6: CALL(6); break;            \
    case 7: CALL(7); break;            \
    case 8: CALL(8); break;            \
    default: break;                    \
  }

// ---------------------------------------------------------------- tile bodies

// x = 0, rhat = r, p = v = 0; ||r||^2
template <int B, class T>
__device__ __forceinline__ void init_tile(const BInst<T>& I, int tile, T (&part)[1]) {
  const int row = tile * kTileRows + static_cast<int>(threadIdx.x);
  if (row >= I.nrows) return;
  const int64_t o = static_cast<int64_t>(row) * B;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const T ri = I.r[o + i];
    I.rhat[o + i] = ri;
    I.p[o + i] = T(0);
    I.v[o + i] = T(0);
    I.x[o + i] = T(0);
    part[0] += ri * ri;
  }
}

// y = D^-1 u for the B values of block row `row`
template <int B, class T>
__device__ __forceinline__ void jacobi_row(const T* __restrict__ dinv, int row, const T (&u)[B], T* __restrict__ y) {
  const T* d = dinv + static_cast<int64_t>(row) * B * B;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < B; ++j) acc += d[i * B + j] * u[j];
    y[i] = acc;
  }
}

// (1) p = r + beta (p - omega v);  phat = D^-1 p
template <int B, class T>
__device__ __forceinline__ void p_tile(const BInst<T>& I, int tile, T beta, T omega) {
  const int row = tile * kTileRows + static_cast<int>(threadIdx.x);
  if (row >= I.nrows) return;
  const int64_t o = static_cast<int64_t>(row) * B;
  T pv[B];
#pragma unroll
  for (int i = 0; i < B; ++i) {
    pv[i] = I.r[o + i] + beta * (I.p[o + i] - omega * I.v[o + i]);
    I.p[o + i] = pv[i];
  }
  jacobi_row<B, T>(I.dinv, row, pv, I.phat + o);
}

// (2) v = A phat; <rhat, v>    (4) t = A shat; <t, s>, <t, t>
template <int B, class T, bool kOmega>
__device__ __forceinline__ void spmv_tile(const BInst<T>& I, int tile, T (&part)[2]) {
  const int warp = static_cast<int>(threadIdx.x) >> 5, lane = static_cast<int>(threadIdx.x) & 31;
  const int64_t sl = static_cast<int64_t>(tile) * kTileWarps + warp;
  if (sl >= I.S.nslices) return;  // warp-uniform
  T y[B];
  sell_lane_rows<B, T, T>(I.S, sl, lane, I.vals, kOmega ? I.shat : I.phat, y);
  const int64_t br = sl * 32 + lane;
  if (br >= I.nrows) return;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const T yt = y[i];
    if constexpr (kOmega) {
      I.t[br * B + i] = yt;
      part[0] += yt * I.s[br * B + i];
      part[1] += yt * yt;
    } else {
      I.v[br * B + i] = yt;
      part[0] += I.rhat[br * B + i] * yt;
    }
  }
}

// (3) s = r - alpha v;  shat = D^-1 s
template <int B, class T>
__device__ __forceinline__ void s_tile(const BInst<T>& I, int tile, T alpha) {
  const int row = tile * kTileRows + static_cast<int>(threadIdx.x);
  if (row >= I.nrows) return;
  const int64_t o = static_cast<int64_t>(row) * B;
  T sv[B];
#pragma unroll
  for (int i = 0; i < B; ++i) {
    sv[i] = I.r[o + i] - alpha * I.v[o + i];
    I.s[o + i] = sv[i];
  }
  jacobi_row<B, T>(I.dinv, row, sv, I.shat + o);
}

// (5) x += alpha phat + omega shat;  r = s - omega t;  ||r||^2, <rhat, r>
template <int B, class T>
__device__ __forceinline__ void xr_tile(const BInst<T>& I, int tile, T alpha, T omega, T (&part)[2]) {
  const int row = tile * kTileRows + static_cast<int>(threadIdx.x);
  if (row >= I.nrows) return;
  const int64_t o = static_cast<int64_t>(row) * B;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    I.x[o + i] = I.x[o + i] + alpha * I.phat[o + i] + omega * I.shat[o + i];
    const T ri = I.s[o + i] - omega * I.t[o + i];
    I.r[o + i] = ri;
    part[0] += ri * ri;
    part[1] += I.rhat[o + i] * ri;
  }
}

// ---------------------------------------------------------------- kernels

template <class T>
__global__ void __launch_bounds__(kTileRows) k_bt_init(const BLane<T>* __restrict__ L) {
  const int n = L->ninit;
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const int2 tl = L->init_tiles[k];
    const BInst<T> I = L->inst[tl.x];
    T part[1] = {T(0)};
#define DC_CALL(B) init_tile<B, T>(I, tl.y, part)
    DC_BT_DISPATCH(I.bs, DC_CALL)
#undef DC_CALL
    double tot[1];
    if (tile_sum<1>(part, tot, L->part + static_cast<int64_t>(I.first_tile) * 2, tl.y, I.ntiles, L->cnt + tl.x)) {
      double* sc = L->sc + static_cast<int64_t>(tl.x) * KS_COUNT;
      const double rr = tot[0];
      sc[KS_RR] = rr;
      sc[KS_RR0] = rr;
      sc[KS_RHO] = rr;
      sc[KS_RHONEW] = rr;
      sc[KS_ALPHA] = 1.0;
      sc[KS_OMEGA] = 1.0;
      sc[KS_BETA] = 1.0;
      sc[KS_TARGET] = I.rel * I.rel * rr;
      sc[KS_ITER] = 0.0;
      sc[KS_DONE] = !isfinite(rr) ? kDoneNonFinite : (rr == 0.0 ? kDoneConverged : 0.0);
    }
  }
}

template <class T>
__global__ void __launch_bounds__(kTileRows) k_bt_p(const BLane<T>* __restrict__ L) {
  const int n = L->ntiles;
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const int2 tl = L->tiles[k];
    const double* sc = L->sc + static_cast<int64_t>(tl.x) * KS_COUNT;
    if (sc[KS_DONE] != 0.0) continue;  // uniform over the block
    const BInst<T> I = L->inst[tl.x];
    const T beta = static_cast<T>(sc[KS_BETA]), omega = static_cast<T>(sc[KS_OMEGA]);
#define DC_CALL(B) p_tile<B, T>(I, tl.y, beta, omega)
    DC_BT_DISPATCH(I.bs, DC_CALL)
#undef DC_CALL
  }
}

template <class T>
__global__ void __launch_bounds__(kTileRows) k_bt_rv(const BLane<T>* __restrict__ L) {
  const int n = L->ntiles;
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const int2 tl = L->tiles[k];
    double* sc = L->sc + static_cast<int64_t>(tl.x) * KS_COUNT;
    if (sc[KS_DONE] != 0.0) continue;
    const BInst<T> I = L->inst[tl.x];
    T part[2] = {T(0), T(0)};
#define DC_CALL(B) spmv_tile<B, T, false>(I, tl.y, part)
    DC_BT_DISPATCH(I.bs, DC_CALL)
#undef DC_CALL
    const T p1[1] = {part[0]};
    double tot[1];
    if (tile_sum<1>(p1, tot, L->part + static_cast<int64_t>(I.first_tile) * 2, tl.y, I.ntiles, L->cnt + tl.x)) {
      const double rv = tot[0];
      sc[KS_RV] = rv;
      const double a = sc[KS_RHO] / rv;
      if (!isfinite(rv)) sc[KS_DONE] = kDoneNonFinite;
      else if (rv == 0.0 || !isfinite(a)) sc[KS_DONE] = kDoneBreakdown;
      sc[KS_ALPHA] = isfinite(a) ? a : 0.0;
    }
  }
}

template <class T>
__global__ void __launch_bounds__(kTileRows) k_bt_s(const BLane<T>* __restrict__ L) {
  const int n = L->ntiles;
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const int2 tl = L->tiles[k];
    const double* sc = L->sc + static_cast<int64_t>(tl.x) * KS_COUNT;
    if (sc[KS_DONE] != 0.0) continue;
    const BInst<T> I = L->inst[tl.x];
    const T alpha = static_cast<T>(sc[KS_ALPHA]);
#define DC_CALL(B) s_tile<B, T>(I, tl.y, alpha)
    DC_BT_DISPATCH(I.bs, DC_CALL)
#undef DC_CALL
  }
}

template <class T>
__global__ void __launch_bounds__(kTileRows) k_bt_omega(const BLane<T>* __restrict__ L) {
  const int n = L->ntiles;
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const int2 tl = L->tiles[k];
    double* sc = L->sc + static_cast<int64_t>(tl.x) * KS_COUNT;
    if (sc[KS_DONE] != 0.0) continue;
    const BInst<T> I = L->inst[tl.x];
    T part[2] = {T(0), T(0)};
#define DC_CALL(B) spmv_tile<B, T, true>(I, tl.y, part)
    DC_BT_DISPATCH(I.bs, DC_CALL)
#undef DC_CALL
    double tot[2];
    if (tile_sum<2>(part, tot, L->part + static_cast<int64_t>(I.first_tile) * 2, tl.y, I.ntiles, L->cnt + tl.x)) {
      sc[KS_TS] = tot[0];
      sc[KS_TT] = tot[1];
      double w = tot[1] != 0.0 ? tot[0] / tot[1] : 0.0;
      if (!isfinite(w)) {
        sc[KS_DONE] = kDoneNonFinite;
        w = 0.0;
      }
      sc[KS_OMEGA] = w;
    }
  }
}

template <class T>
__global__ void __launch_bounds__(kTileRows) k_bt_xr(const BLane<T>* __restrict__ L) {
  const int n = L->ntiles;
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const int2 tl = L->tiles[k];
    double* sc = L->sc + static_cast<int64_t>(tl.x) * KS_COUNT;
    if (sc[KS_DONE] != 0.0) continue;
    const BInst<T> I = L->inst[tl.x];
    const T alpha = static_cast<T>(sc[KS_ALPHA]), omega = static_cast<T>(sc[KS_OMEGA]);
    T part[2] = {T(0), T(0)};
#define DC_CALL(B) xr_tile<B, T>(I, tl.y, alpha, omega, part)
    DC_BT_DISPATCH(I.bs, DC_CALL)
#undef DC_CALL
    double tot[2];
    if (tile_sum<2>(part, tot, L->part + static_cast<int64_t>(I.first_tile) * 2, tl.y, I.ntiles, L->cnt + tl.x)) {
      const double rr = tot[0], rho_new = tot[1];
      sc[KS_RR] = rr;
      sc[KS_RHONEW] = rho_new;
      sc[KS_ITER] += 1.0;
      if (!isfinite(rr) || !isfinite(rho_new)) {
        sc[KS_DONE] = kDoneNonFinite;
      } else if (rr <= sc[KS_TARGET]) {
        sc[KS_DONE] = kDoneConverged;
      } else {
        const double beta = (rho_new / sc[KS_RHO]) * (sc[KS_ALPHA] / sc[KS_OMEGA]);
        if (rho_new == 0.0 || sc[KS_OMEGA] == 0.0 || !isfinite(beta)) {
          sc[KS_DONE] = kDoneBreakdown;
        } else {
          sc[KS_BETA] = beta;
          sc[KS_RHO] = rho_new;
          if (sc[KS_ITER] >= static_cast<double>(I.max_it)) sc[KS_DONE] = kDoneMaxIt;
        }
      }
    }
  }
}

#undef DC_BT_DISPATCH

// ---------------------------------------------------------------- host side

struct Request {
  int prec = 0;  // 0: fp32, 1: fp64
  BatchSystem<float> s32{};
  BatchSystem<double> s64{};
  cudaEvent_t ready = nullptr;
  double rel = 0.0;
  int max_it = 0;
  bool done = false;
  int status = 0;
  int iters = 0;
  std::string error;
  std::condition_variable cv;  // the caller waits on it (with the batcher's mutex)
};

template <class T>
void free_host(T*& p) {
  if (p) cudaFreeHost(p);
  p = nullptr;
}

template <class T>
void alloc_host(T*& p, size_t n) {
  free_host(p);
  cuda_check(cudaMallocHost(reinterpret_cast<void**>(&p), std::max<size_t>(n, 1) * sizeof(T)), "cudaMallocHost");
}

inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// One precision's slots, table and captured graphs.  Only the batch thread touches a lane
// after construction.
//
// The table is one device buffer, uploaded by one copy per replay: the header (BLane), the
// slot descriptors, then the tiles of all active instances followed by the tiles of the
// instances admitted for this replay.  Graphs are captured for a few grid sizes (the
// kernels read the header at the table's start), and an autotuner picks the grid per batch
// size: a replay of t tiles falls in bucket floor(log2 t); a bucket first times each grid
// that leaves at most 64 tiles to a block on kTuneSamples replays (CUDA events around the
// graph launch), then runs the one with the least mean time.  The batch shares the device
// with the other simulations' kernels, so the fastest grid depends on the load as well as
// on the size; the results do not depend on the grid (the tile decomposition is fixed).
template <class T>
struct Lane {
  int max_slots = 0;
  int grid_full = 0;
  cudaStream_t stream = nullptr;
  std::vector<Request*> slot;  // null: free
  std::vector<char> fresh;     // admitted since the last replay
  DeviceBuffer<unsigned char> table;
  unsigned char* h_table = nullptr;
  size_t off_inst = 0, off_tiles = 0;
  size_t tile_cap = 0;  // run + init tiles the table holds
  DeviceBuffer<double> sc, part;
  DeviceBuffer<unsigned int> cnt;
  double* h_sc = nullptr;
  struct GridGraphs {
    int grid;
    cudaGraphExec_t exec[kNumChunks];  // kChunks[c] iterations
  };
  std::vector<GridGraphs> graphs;  // ascending grid
  // chunk length: running mean of the lane's solve lengths, and each slot's iterations so far
  double mean_iters = 8.0;
  std::vector<int> slot_iters;

  static constexpr int kBuckets = 24, kTuneSamples = 3, kMaxGrids = 3;
  struct Bucket {
    double ms[kMaxGrids] = {};
    int n[kMaxGrids] = {};
    int chosen = -1;  // index into graphs once tuned
  };
  std::array<Bucket, kBuckets> tune{};
  cudaEvent_t tev[2] = {nullptr, nullptr};
  int timed_bucket = -1, timed_graph = -1, timed_tiles = 0;  // the timed replay in flight
  int timed_chunk = kChunks[kNumChunks - 1];                   // its iterations (times are per iteration)

  const BLane<T>* dev_header() const { return reinterpret_cast<const BLane<T>*>(table.get()); }

  // a candidate grid for t tiles: at most 64 tiles to a block (the largest grid always)
  bool candidate(int i, int tiles) const {
    return 64 * static_cast<int64_t>(graphs[i].grid) >= tiles || i + 1 == static_cast<int>(graphs.size());
  }

  // graph index for a replay of `tiles` tiles; sets timed_* when this replay is a tuning
  // sample (the least-sampled candidate of an untuned bucket)
  int pick_graph(int tiles) {
    int b = 0;
    while (b + 1 < kBuckets && (2 << b) <= tiles) ++b;
    const Bucket& k = tune[b];
    timed_bucket = timed_graph = -1;
    if (k.chosen >= 0) return k.chosen;
    int best = -1;
    for (int i = 0; i < static_cast<int>(graphs.size()); ++i)
      if (candidate(i, tiles) && (best < 0 || k.n[i] < k.n[best])) best = i;
    timed_bucket = b;
    timed_graph = best;
    timed_tiles = tiles;
    return best;
  }

  // after the stream has been synchronised (under the batcher's mutex): books the timed
  // replay's duration, and settles the bucket on its fastest candidate once every candidate
  // has kTuneSamples samples
  void book_timing() {
    if (timed_bucket < 0) return;
    Bucket& k = tune[timed_bucket];
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, tev[0], tev[1]) == cudaSuccess) {
      k.ms[timed_graph] += ms / timed_chunk;
      k.n[timed_graph] += 1;
    } else {
      cudaGetLastError();  // an unreadable sample is dropped
    }
    bool complete = true;
    int best = -1;
    for (int i = 0; i < static_cast<int>(graphs.size()); ++i) {
      if (!candidate(i, timed_tiles)) continue;
      if (k.n[i] < kTuneSamples) complete = false;
      else if (best < 0 || k.ms[i] / k.n[i] < k.ms[best] / k.n[best]) best = i;
    }
    if (complete && best >= 0) k.chosen = best;
    timed_bucket = timed_graph = -1;
  }

  // the tuned grids as JSON: {"<first tile count of the bucket>": grid, ...}
  std::string tuning_json() const {
    std::string out = "{";
    for (int b = 0; b < kBuckets; ++b)
      if (tune[b].chosen >= 0) {
        if (out.size() > 1) out += ", ";
        out += "\"" + std::to_string(1 << b) + "\": " + std::to_string(graphs[tune[b].chosen].grid);
      }
    return out + "}";
  }

  void create(int slots, int full_grid, cudaStream_t s) {
    max_slots = slots;
    grid_full = full_grid;
    stream = s;
    slot.assign(slots, nullptr);
    fresh.assign(slots, 0);
    slot_iters.assign(slots, 0);
    sc.resize(static_cast<size_t>(slots) * KS_COUNT);
    cnt.resize(slots);
    cuda_check(cudaMemsetAsync(cnt.get(), 0, slots * sizeof(unsigned int), stream), "memset");
    cuda_check(cudaMemsetAsync(sc.get(), 0, static_cast<size_t>(slots) * KS_COUNT * sizeof(double), stream), "memset");
    alloc_host(h_sc, static_cast<size_t>(slots) * KS_COUNT);
    for (auto& e : tev) cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    off_inst = round_up(sizeof(BLane<T>), 256);
    off_tiles = round_up(off_inst + static_cast<size_t>(slots) * sizeof(BInst<T>), 256);
    reserve(2048);
  }

  void drop_graphs() {
    for (auto& g : graphs)
      for (auto& e : g.exec)
        if (e) cudaGraphExecDestroy(e);
    graphs.clear();
  }

  void destroy() {
    drop_graphs();
    for (auto& e : tev)
      if (e) cudaEventDestroy(e);
    tev[0] = tev[1] = nullptr;
    free_host(h_table);
    free_host(h_sc);
  }

  // kChunks[c] iterations of the five phases at each grid size (called with the stream idle)
  void capture() {
    drop_graphs();
    const BLane<T>* L = dev_header();
    for (int grid : {32, 128, grid_full}) {
      if (grid > grid_full || (!graphs.empty() && graphs.back().grid >= grid)) continue;
      GridGraphs gg{grid, {}};
      graphs.push_back(gg);
      for (int c = 0; c < kNumChunks; ++c) {
        cudaGraph_t g = nullptr;
        cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        for (int k = 0; k < kChunks[c]; ++k) {
          k_bt_p<T><<<grid, kTileRows, 0, stream>>>(L);
          k_bt_rv<T><<<grid, kTileRows, 0, stream>>>(L);
          k_bt_s<T><<<grid, kTileRows, 0, stream>>>(L);
          k_bt_omega<T><<<grid, kTileRows, 0, stream>>>(L);
          k_bt_xr<T><<<grid, kTileRows, 0, stream>>>(L);
        }
        cuda_check(cudaStreamEndCapture(stream, &g), "cudaStreamEndCapture");
        cuda_check(cudaGetLastError(), "batched BiCGSTAB capture");
        const cudaError_t e = cudaGraphInstantiate(&graphs.back().exec[c], g, 0);
        cudaGraphDestroy(g);
        cuda_check(e, "cudaGraphInstantiate");
      }
    }
  }

  // chunk index of the next replay: the shortest captured length that covers the iterations
  // the active instance closest to convergence is expected to need (the lane's mean solve
  // length less the iterations it has run, at least one)
  int pick_chunk() const {
    double need = 1e30;
    for (int k = 0; k < max_slots; ++k)
      if (slot[k]) need = std::min(need, std::max(1.0, mean_iters - slot_iters[k]));
    for (int c = 0; c < kNumChunks; ++c)
      if (kChunks[c] >= need) return c;
    return kNumChunks - 1;
  }

  // room for n tiles (run + init) in the table (called with the stream idle); the table
  // moves, so the graphs are captured again
  void reserve(size_t n) {
    if (n <= tile_cap) return;
    size_t cap = std::max<size_t>(tile_cap, 2048);
    while (cap < n) cap *= 2;
    const size_t bytes = off_tiles + cap * sizeof(int2);
    table.resize(bytes);
    alloc_host(h_table, bytes);
    part.resize(cap * 2);
    tile_cap = cap;
    capture();
  }

  int active() const {
    int a = 0;
    for (const Request* q : slot) a += q != nullptr;
    return a;
  }

  bool admit(Request* q) {
    for (int k = 0; k < max_slots; ++k)
      if (!slot[k]) {
        slot[k] = q;
        fresh[k] = 1;
        slot_iters[k] = 0;
        return true;
      }
    return false;
  }

  static const BatchSystem<T>& system(const Request* q) {
    if constexpr (std::is_same_v<T, float>) return q->s32;
    else return q->s64;
  }

  int nt = 0, ni = 0, top = 0;  // the next replay's run tiles, init tiles and slot bound

  // sizes the next replay and makes room for it (with the stream idle: a larger table is a
  // new allocation and new graphs)
  void plan() {
    nt = ni = top = 0;
    for (int k = 0; k < max_slots; ++k) {
      if (!slot[k]) continue;
      const int tk = (system(slot[k]).nrows + kTileRows - 1) / kTileRows;
      nt += tk;
      if (fresh[k]) ni += tk;
      top = k + 1;
    }
    reserve(static_cast<size_t>(nt) + ni);
  }

  // enqueues the planned replay (the table upload, the new instances' initialisation, the
  // graph, the scalars' download) on the stream; returns the kernels launched
  long long enqueue() {
    BInst<T>* hi = reinterpret_cast<BInst<T>*>(h_table + off_inst);
    int2* ht = reinterpret_cast<int2*>(h_table + off_tiles);
    int t = 0, it = nt;
    for (int k = 0; k < top; ++k) {
      Request* q = slot[k];
      if (!q) continue;
      const BatchSystem<T>& y = system(q);
      BInst<T>& d = hi[k];
      d.nrows = y.nrows;
      d.bs = y.bs;
      d.ntiles = (y.nrows + kTileRows - 1) / kTileRows;
      d.first_tile = t;
      d.rel = q->rel;
      d.max_it = q->max_it;
      d.pad = 0;
      d.S = y.S;
      d.vals = y.vals;
      d.dinv = y.dinv;
      d.x = y.x; d.r = y.r; d.rhat = y.rhat; d.p = y.p; d.v = y.v; d.s = y.s; d.t = y.t;
      d.phat = y.phat; d.shat = y.shat;
      for (int j = 0; j < d.ntiles; ++j) ht[t + j] = make_int2(k, j);
      if (fresh[k]) {
        for (int j = 0; j < d.ntiles; ++j) ht[it + j] = make_int2(k, j);
        it += d.ntiles;
        cuda_check(cudaStreamWaitEvent(stream, q->ready, 0), "cudaStreamWaitEvent");
        fresh[k] = 0;
      }
      t += d.ntiles;
    }
    const int2* dt = reinterpret_cast<const int2*>(table.get() + off_tiles);
    *reinterpret_cast<BLane<T>*>(h_table) =
        BLane<T>{nt, ni, dt, dt + nt, reinterpret_cast<const BInst<T>*>(table.get() + off_inst), sc.get(), part.get(),
                 cnt.get()};
    cuda_check(cudaMemcpyAsync(table.get(), h_table, off_tiles + static_cast<size_t>(nt + ni) * sizeof(int2),
                               cudaMemcpyHostToDevice, stream), "upload");
    long long launched = 0;
    if (ni) {
      k_bt_init<T><<<std::min(ni, grid_full), kTileRows, 0, stream>>>(dev_header());
      cuda_check(cudaGetLastError(), "batched BiCGSTAB init");
      ++launched;
    }
    const int ci = pick_chunk();
    const int gi = pick_graph(nt);
    timed_chunk = kChunks[ci];
    if (timed_bucket >= 0) cuda_check(cudaEventRecord(tev[0], stream), "cudaEventRecord");
    cuda_check(cudaGraphLaunch(graphs[gi].exec[ci], stream), "cudaGraphLaunch");
    if (timed_bucket >= 0) cuda_check(cudaEventRecord(tev[1], stream), "cudaEventRecord");
    launched += static_cast<long long>(kChunks[ci]) * kPhases;
    cuda_check(cudaMemcpyAsync(h_sc, sc.get(), static_cast<size_t>(top) * KS_COUNT * sizeof(double),
                               cudaMemcpyDeviceToHost, stream), "download");
    return launched;
  }

  // after the stream has been synchronised: hands back the instances that are done
  void retire(std::vector<Request*>& finished, BatchStats& st) {
    for (int k = 0; k < max_slots; ++k) {
      Request* q = slot[k];
      if (!q) continue;
      const double* s = h_sc + static_cast<int64_t>(k) * KS_COUNT;
      const double d = s[KS_DONE];
      slot_iters[k] = static_cast<int>(s[KS_ITER]);
      if (d == 0.0) continue;
      q->iters = static_cast<int>(s[KS_ITER]);
      mean_iters = 0.8 * mean_iters + 0.2 * q->iters;
      q->status = d == kDoneConverged ? 0 : (d == kDoneMaxIt ? 3 : 1);
      st.solves += 1;
      st.iterations += q->iters;
      finished.push_back(q);
      slot[k] = nullptr;
    }
  }

  // a failure: every request the lane holds ends with `why`
  void fail_all(const std::string& why) {
    for (Request*& q : slot)
      if (q) {
        q->error = why;
        q->done = true;
        q->cv.notify_one();
        q = nullptr;
      }
  }
};

}  // namespace

struct KrylovBatcher::Impl {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::condition_variable cv_work;
  std::deque<Request*> pending;
  bool stop = false;
  std::string fatal;  // a CUDA failure of the batch thread: later solves fail with it
  BatchStats st;
  Lane<float> l32;
  Lane<double> l64;
  std::thread th;

  void loop();
  template <class T>
  int submit(const BatchSystem<T>& sys, cudaStream_t caller, double rel, int max_it, int* iters);
};

KrylovBatcher::KrylovBatcher(int device, int max_slots) : impl_(std::make_unique<Impl>()) {
  if (max_slots < 1 || max_slots > 1024) throw std::invalid_argument("batch slots must be in [1, 1024]");
  Impl& m = *impl_;
  m.device = device;
  cuda_check(cudaSetDevice(device), "cudaSetDevice");
  int sms = 0;
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
  // the batch is on every served simulation's critical path: its blocks go first
  int prio_low = 0, prio_high = 0;
  cuda_check(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high), "cudaDeviceGetStreamPriorityRange");
  cuda_check(cudaStreamCreateWithPriority(&m.stream, cudaStreamNonBlocking, prio_high), "cudaStreamCreate");
  try {
    // at most four 256-thread blocks per SM walk the tile table
    m.l32.create(max_slots, 4 * sms, m.stream);
    m.l64.create(max_slots, 4 * sms, m.stream);
    cuda_check(cudaStreamSynchronize(m.stream), "cudaStreamSynchronize");
  } catch (...) {
    m.l32.destroy();
    m.l64.destroy();
    cudaStreamDestroy(m.stream);
    throw;
  }
  m.th = std::thread([&m] { m.loop(); });
}

KrylovBatcher::~KrylovBatcher() {
  Impl& m = *impl_;
  {
    std::lock_guard<std::mutex> lk(m.mu);
    m.stop = true;
  }
  m.cv_work.notify_all();
  if (m.th.joinable()) m.th.join();
  cudaStreamSynchronize(m.stream);
  m.l32.destroy();
  m.l64.destroy();
  cudaStreamDestroy(m.stream);
}

BatchStats KrylovBatcher::stats() const {
  std::lock_guard<std::mutex> lk(impl_->mu);
  return impl_->st;
}

std::string KrylovBatcher::tuning() const {
  std::lock_guard<std::mutex> lk(impl_->mu);
  return "{\"fp32\": " + impl_->l32.tuning_json() + ", \"fp64\": " + impl_->l64.tuning_json() + "}";
}

int KrylovBatcher::solve(const BatchSystem<float>& sys, cudaStream_t caller, double rel, int max_it, int* iters) {
  return impl_->submit(sys, caller, rel, max_it, iters);
}
int KrylovBatcher::solve(const BatchSystem<double>& sys, cudaStream_t caller, double rel, int max_it, int* iters) {
  return impl_->submit(sys, caller, rel, max_it, iters);
}

namespace {
// the calling thread's event that marks where the batch may start on its stream
struct ReadyEvent {
  cudaEvent_t e = nullptr;
  ~ReadyEvent() {
    if (e) cudaEventDestroy(e);
  }
};
}  // namespace

template <class T>
int KrylovBatcher::Impl::submit(const BatchSystem<T>& sys, cudaStream_t caller, double rel, int max_it, int* iters) {
  *iters = 0;
  if (sys.bs < 1 || sys.bs > 8) throw std::invalid_argument("batched BiCGSTAB: block size must be in [1, 8]");
  if (sys.nrows < 0) throw std::invalid_argument("batched BiCGSTAB: negative row count");
  if (sys.nrows == 0) return 0;
  thread_local ReadyEvent ev;
  if (!ev.e) cuda_check(cudaEventCreateWithFlags(&ev.e, cudaEventDisableTiming), "cudaEventCreate");
  cuda_check(cudaEventRecord(ev.e, caller), "cudaEventRecord");
  Request q;
  if constexpr (std::is_same_v<T, float>) {
    q.prec = 0;
    q.s32 = sys;
  } else {
    q.prec = 1;
    q.s64 = sys;
  }
  q.ready = ev.e;
  q.rel = rel;
  q.max_it = std::max(max_it, 1);
  const auto t0 = std::chrono::steady_clock::now();
  std::unique_lock<std::mutex> lk(mu);
  if (!fatal.empty()) throw CudaError(fatal);
  pending.push_back(&q);
  cv_work.notify_one();
  q.cv.wait(lk, [&] { return q.done; });
  st.wait_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (!q.error.empty()) throw CudaError(q.error);
  *iters = q.iters;
  return q.status;
}

void KrylovBatcher::Impl::loop() {
  cudaSetDevice(device);
  std::vector<Request*> finished;
  try {
    while (true) {
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || !pending.empty() || l32.active() > 0 || l64.active() > 0; });
        if (pending.empty() && l32.active() == 0 && l64.active() == 0) {
          if (stop) return;
          continue;
        }
        // admit in arrival order while slots are free
        for (auto it = pending.begin(); it != pending.end();) {
          Request* q = *it;
          const bool ok = q->prec == 0 ? l32.admit(q) : l64.admit(q);
          it = ok ? pending.erase(it) : std::next(it);
        }
      }
      const auto t0 = std::chrono::steady_clock::now();
      const int a32 = l32.active(), a64 = l64.active();
      long long launched = 0;
      if (a32) l32.plan();
      if (a64) l64.plan();
      if (a32) launched += l32.enqueue();
      if (a64) launched += l64.enqueue();
      count_launches(launched);
      cuda_check(cudaStreamSynchronize(stream), "batched BiCGSTAB");
      finished.clear();
      std::lock_guard<std::mutex> lk(mu);
      st.replay_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      st.replays += (a32 > 0) + (a64 > 0);
      st.slot_replays += a32 + a64;
      st.max_active = std::max<int32_t>(st.max_active, a32 + a64);
      l32.book_timing();
      l64.book_timing();
      l32.retire(finished, st);
      l64.retire(finished, st);
      // under the lock: a caller returns (and destroys its request) only after taking it
      for (Request* q : finished) {
        q->done = true;
        q->cv.notify_one();
      }
    }
  } catch (const std::exception& e) {
    // nothing of the batch may still run on the callers' buffers when they resume
    cudaStreamSynchronize(stream);
    std::lock_guard<std::mutex> lk(mu);
    fatal = std::string("batched BiCGSTAB: ") + e.what();
    for (Request* q : pending) {
      q->error = fatal;
      q->done = true;
      q->cv.notify_one();
    }
    pending.clear();
    l32.fail_all(fatal);
    l64.fail_all(fatal);
  }
}

}  // namespace dcgpu
