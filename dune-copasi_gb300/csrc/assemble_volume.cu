// Volume assembly kernels: residual and analytic Jacobian of the mass and stiffness
// forms (dune/copasi/model/diffusion_reaction/local_operator.hh:417-491, 541-707).
#include <cstdio>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "assemble.cuh"
#include "interp.cuh"
#include "linalg.cuh"
#include "volume_kernel.cuh"

namespace dcgpu {

namespace {

using namespace vk;

// The library's Spec of the volume element body (volume_kernel.cuh): term lists and
// program outputs read from device memory, the program run by the bytecode interpreter
// with its register file in shared memory.
struct InterpSpec {
  static constexpr bool kUnrollPoints = false;
  __device__ __forceinline__ static int n_res(const VolumeParams& P, bool) { return P.n_res_terms; }
  __device__ __forceinline__ static Term res(const VolumeParams& P, bool, int t) { return P.res_terms[t]; }
  __device__ __forceinline__ static int n_jac(const VolumeParams& P) { return P.n_jac_terms; }
  __device__ __forceinline__ static Term jac(const VolumeParams& P, int t) { return P.jac_terms[t]; }
  __device__ __forceinline__ static int out(const VolumeParams& P, bool, int i) { return P.prog.outputs[i]; }
  __device__ __forceinline__ static int n_slots(const VolumeParams& P) { return P.n_slots; }
  __device__ __forceinline__ static bool all_mass(const VolumeParams& P) { return P.all_mass != 0; }
  __device__ __forceinline__ static bool need_grad(const VolumeParams& P) { return P.need_grad != 0; }
  __device__ __forceinline__ static bool has_flux(const VolumeParams& P) { return P.has_flux != 0; }
  __device__ __forceinline__ static bool need_pos(const VolumeParams& P) { return P.need_pos != 0; }
  __device__ __forceinline__ static bool need_vol(const VolumeParams& P) { return P.need_vol != 0; }
  __device__ __forceinline__ static int coef_bound(const VolumeParams&, int ncoef) { return ncoef; }
  template <class F>
  __device__ __forceinline__ static StridedCast<F, float> as_float(const Strided<F>& c) {
    return StridedCast<F, float>{c.p, c.stride};
  }
  template <int DIM, int NS, class F, class Regs>
  __device__ __forceinline__ static void run(const VolumeParams& P, bool, Regs R, const F (&u)[NS],
                                             const F (&g)[NS][DIM], const F (&xq)[DIM], F t, F vol) {
    for (int i = 0; i < P.prog.ninputs; ++i)
      R[i] = volume_input<DIM, NS, F>(P.prog.inputs[i], u, g, xq, t, vol, P.species_offset);
    run_program<F>(P.prog, P.tables, R);
  }
};

// One thread per cell; the interpreter's registers and the Jacobian coefficients are
// per-thread slices of dynamic shared memory (sized by the launcher from the program's
// registers and the term list).
template <int DIM, int NS, class F>
__global__ void __launch_bounds__(128) k_volume(const VolumeParams P, const int begin, const int end,
                                                const int mode) {
  const int k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;
  extern __shared__ __align__(16) unsigned char volume_smem[];
  F* const smem = reinterpret_cast<F*>(volume_smem);
  const Strided<F> R{smem + threadIdx.x, static_cast<int>(blockDim.x)};
  const Strided<F> coef{smem + static_cast<int64_t>(P.prog.nregs) * blockDim.x + threadIdx.x,
                        static_cast<int>(blockDim.x)};
  volume_element<DIM, NS, F, InterpSpec, 0>(P, k, mode, R, coef);
}

// sum of v[list[i] * stride + col] for i in [i0, i1), added in ascending i.  The list
// entries and the values are fetched eight at a time as independent loads (the plain loop
// is a chain of dependent list -> value loads, latency-bound); the sum order is unchanged.
// Used by the block gather (nine-entry element matrices, long lists); the node gather's
// short lists measured faster with the plain loop.
template <class E>
__device__ __forceinline__ E gather_sum(int64_t i0, int64_t i1, const int32_t* __restrict__ list,
                                        const E* __restrict__ v, unsigned stride, unsigned col) {
  constexpr int kBatch = 8;
  E acc = E(0);
  for (int64_t i = i0; i < i1; i += kBatch) {
    int32_t idx[kBatch];
    E val[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) idx[u] = i + u < i1 ? list[i + u] : 0;
#pragma unroll
    for (int u = 0; u < kBatch; ++u)
      val[u] = i + u < i1 ? v[static_cast<int64_t>(idx[u]) * stride + col] : E(0);
#pragma unroll
    for (int u = 0; u < kBatch; ++u)
      if (i + u < i1) acc += val[u];
  }
  return acc;
}

// r[node, s] += sum of the element residual entries of the node's (element, vertex) list;
// a thread per (node, species), species fastest, 32-bit index arithmetic
__global__ void k_gather_residual(double* __restrict__ r, int bs, unsigned ns, int64_t node_begin, unsigned ntotal,
                                  const int64_t* __restrict__ ptr, const int32_t* __restrict__ list,
                                  const double* __restrict__ er) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntotal) return;
  const unsigned n = t / ns, s = t - n * ns;
  double acc = 0.0;
  for (int64_t i = ptr[n]; i < ptr[n + 1]; ++i) acc += er[static_cast<int64_t>(list[i]) * ns + s];
  r[(node_begin + n) * bs + s] += acc;
}

// J[block, slot position] += sum of the element Jacobian values (type E) of the block's
// (element, local pair) list.  A thread per (block, slot), slot fastest, so the threads of a
// warp read neighbouring element values and write neighbouring entries; 32-bit index
// arithmetic (the host checks nblocks * nslot < 2^32; 64-bit division is a long routine).
template <class E>
__global__ void k_gather_jacobian(double* __restrict__ J, int bs2, unsigned nslot, const int32_t* __restrict__ slot_pos,
                                  int64_t block_begin, unsigned ntotal, const int64_t* __restrict__ ptr,
                                  const int32_t* __restrict__ list, const E* __restrict__ ej, const JacobianGatherOut o) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntotal) return;
  const unsigned b = t / nslot, m = t - b * nslot;
  const E acc = gather_sum<E>(ptr[b], ptr[b + 1], list, ej, nslot, m);
  const int64_t blk = block_begin + b;
  const int64_t at = blk * bs2 + slot_pos[m];
  // overwrite: this gather covers every entry of J, so the static operator (or zero) is its
  // base and no separate copy of it into J runs
  const double v = (o.overwrite ? (o.base ? o.base[at] : 0.0) : J[at]) + static_cast<double>(acc);
  J[at] = v;
  if (o.sell) o.sell[sell_value_index(o.sell_bpos[blk], slot_pos[m], bs2)] = static_cast<float>(v);
}

// A gather that covers every block of J when only some entries of a block have dynamic
// terms: a thread per (block, entry), entry fastest; entry e takes the base (static
// operator, or zero) plus, when a dynamic slot feeds it, that slot's element values.  J and
// the fp32 SELL-32 copy are written once, with no copy of the base into J and no
// conversion pass before or after.
struct EntrySlots {
  int8_t slot[64];  // dynamic slot of entry test * bs + trial, or -1
};
template <class E>
__global__ void k_gather_jacobian_full(double* __restrict__ J, unsigned bs2, unsigned nslot, const EntrySlots es,
                                       int64_t block_begin, unsigned ntotal, const int64_t* __restrict__ ptr,
                                       const int32_t* __restrict__ list, const E* __restrict__ ej,
                                       const JacobianGatherOut o) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntotal) return;
  const unsigned b = t / bs2, e = t - b * bs2;
  const int m = es.slot[e];
  const int64_t blk = block_begin + b;
  const int64_t at = blk * bs2 + e;
  double v = o.base ? o.base[at] : 0.0;
  if (m >= 0) v += static_cast<double>(gather_sum<E>(ptr[b], ptr[b + 1], list, ej, nslot, static_cast<unsigned>(m)));
  J[at] = v;
  if (o.sell) o.sell[sell_value_index(o.sell_bpos[blk], e, bs2)] = static_cast<float>(v);
}

// The covering gather with a thread per block of J: the block's (cell, local pair) list is
// read once and each entry's slot values (contiguous in the element record) summed per slot
// in list order, the same order and so the same bits as the per-entry gathers.  The block
// values start from the base (static operator) read through shared memory and go back
// through it, so J's loads and stores are contiguous across the thread block; the fp32
// SELL-32 copy is written from the same values.  BS2 = bs * bs (at most 25 here).
constexpr int kBlockGatherThreads = 128;
template <class E, int BS2>
__global__ void __launch_bounds__(kBlockGatherThreads)
    k_gather_jacobian_blocks(double* __restrict__ J, int nslot, const EntrySlots es, int64_t block_begin,
                             unsigned nblocks, const int64_t* __restrict__ ptr, const int32_t* __restrict__ list,
                             const E* __restrict__ ej, const JacobianGatherOut o) {
  constexpr int SB = BS2 | 1;  // odd stride: the threads' own blocks sit in distinct banks
  __shared__ double stage[kBlockGatherThreads * SB];
  const unsigned b0 = blockIdx.x * kBlockGatherThreads;
  const int nb = static_cast<int>(min(static_cast<unsigned>(kBlockGatherThreads), nblocks - b0));
  const int64_t g0 = (block_begin + b0) * BS2;
  for (int i = threadIdx.x; i < nb * BS2; i += kBlockGatherThreads) {
    const int t = i / BS2, e = i - t * BS2;
    stage[t * SB + e] = o.base ? o.base[g0 + i] : 0.0;
  }
  __syncthreads();
  if (static_cast<int>(threadIdx.x) < nb) {
    const unsigned b = b0 + threadIdx.x;
    E acc[BS2];
#pragma unroll
    for (int m = 0; m < BS2; ++m) acc[m] = E(0);
    const int64_t i0 = ptr[b], i1 = ptr[b + 1];
    constexpr int kBatch = 4;
    for (int64_t i = i0; i < i1; i += kBatch) {
      int32_t idx[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) idx[u] = i + u < i1 ? list[i + u] : 0;
      E val[kBatch][BS2];
#pragma unroll
      for (int u = 0; u < kBatch; ++u)
#pragma unroll
        for (int m = 0; m < BS2; ++m)
          val[u][m] = (m < nslot && i + u < i1) ? ej[static_cast<int64_t>(idx[u]) * nslot + m] : E(0);
#pragma unroll
      for (int u = 0; u < kBatch; ++u)
        if (i + u < i1) {
#pragma unroll
          for (int m = 0; m < BS2; ++m)
            if (m < nslot) acc[m] += val[u][m];
        }
    }
    double* mine = stage + threadIdx.x * SB;
#pragma unroll
    for (int e = 0; e < BS2; ++e) {
      const int m = es.slot[e];
#pragma unroll
      for (int mm = 0; mm < BS2; ++mm)
        if (mm == m) mine[e] += static_cast<double>(acc[mm]);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb * BS2; i += kBlockGatherThreads) {
    const int t = i / BS2, e = i - t * BS2;
    const double v = stage[t * SB + e];
    J[g0 + i] = v;
    if (o.sell) o.sell[sell_value_index(o.sell_bpos[block_begin + b0 + t], e, BS2)] = static_cast<float>(v);
  }
}

// Local residual of one element for coefficients c (residual terms only, both forms).
template <int DIM, int NS>
__device__ void fd_local_residual(const VolumeParams& P, const double (&c)[DIM + 1][NS], const double (&X)[DIM + 1][DIM],
                                  const double (&Bm)[DIM][DIM], const double (&G)[DIM + 1][DIM], double adet,
                                  double vol, double (&rl)[DIM + 1][NS], double* R) {
  constexpr int NL = DIM + 1;
  constexpr int NQ = Rule<DIM>::NQ;
  double g[NS][DIM];
#pragma unroll
  for (int s = 0; s < NS; ++s)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      double acc = 0.0;
#pragma unroll
      for (int a = 0; a < NL; ++a) acc += c[a][s] * G[a][j];
      g[s][j] = acc;
    }
#pragma unroll
  for (int a = 0; a < NL; ++a)
#pragma unroll
    for (int s = 0; s < NS; ++s) rl[a][s] = 0.0;
#pragma unroll 1
  for (int q = 0; q < NQ; ++q) {
    double u[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      double acc = 0.0;
#pragma unroll
      for (int a = 0; a < NL; ++a) acc += c[a][s] * phi<DIM>(q, a);
      u[s] = acc;
    }
    double xq[DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      double acc = X[0][i];
#pragma unroll
      for (int j = 0; j < DIM; ++j) acc += Bm[i][j] * Rule<DIM>::xi(q, j);
      xq[i] = acc;
    }
    const double fq = Rule<DIM>::w(q) * adet;
    for (int i = 0; i < P.prog.ninputs; ++i)
      R[i] = volume_input<DIM, NS>(P.prog.inputs[i], u, g, xq, P.t, vol, P.species_offset);
    run_program<double>(P.prog, P.tables, R);
    const uint8_t* out = P.prog.outputs;
    double scal[NS], flux[NS][DIM];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      scal[s] = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; ++j) flux[s][j] = 0.0;
    }
    for (int t = 0; t < P.n_res_terms; ++t) {
      const Term T = P.res_terms[t];
      const double sc = T.form ? P.ca : P.cm;
      const double o = R[out[T.out]];
      double ut = 0.0, gw[DIM];
#pragma unroll
      for (int s = 0; s < NS; ++s)
        if (s == T.test) ut = u[s];
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        gw[j] = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
          if (s == T.trial) gw[j] = g[s][j];
      }
      double ds = 0.0, df[DIM];
#pragma unroll
      for (int j = 0; j < DIM; ++j) df[j] = 0.0;
      switch (T.kind) {
        case R_REACTION: ds = -o; break;
        case R_STORAGE: ds = ut * o; break;
        case R_VELOCITY:
#pragma unroll
          for (int j = 0; j < DIM; ++j) df[j] = R[out[T.out + j]] * ut;
          break;
        case R_DIFF_SCALAR:
#pragma unroll
          for (int j = 0; j < DIM; ++j) df[j] = -o * gw[j];
          break;
        case R_DIFF_TENSOR:
#pragma unroll
          for (int i = 0; i < DIM; ++i) {
            double acc = 0.0;
#pragma unroll
            for (int j = 0; j < DIM; ++j) acc += R[out[T.out + i * DIM + j]] * gw[j];
            df[i] = -acc;
          }
          break;
        default: break;
      }
#pragma unroll
      for (int s = 0; s < NS; ++s)
        if (s == T.test) {
          scal[s] += sc * ds;
#pragma unroll
          for (int j = 0; j < DIM; ++j) flux[s][j] += sc * df[j];
        }
    }
#pragma unroll
    for (int a = 0; a < NL; ++a) {
      const double pa = phi<DIM>(q, a);
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        double fg = 0.0;
#pragma unroll
        for (int j = 0; j < DIM; ++j) fg += flux[s][j] * G[a][j];
        rl[a][s] += (scal[s] * pa - fg) * fq;
      }
    }
  }
}

// Numerical element Jacobian by forward differences of the local residual,
// delta = eps (1 + |c|) per local coefficient (local_operator.hh:713-765).
template <int DIM, int NS>
__global__ void __launch_bounds__(128) k_volume_fd(const VolumeParams P, const int begin, const int end) {
  constexpr int NL = DIM + 1;
  const int k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;
  int nd[NL];
  double X[NL][DIM];
#pragma unroll
  for (int a = 0; a < NL; ++a) {
    const int v = P.verts[static_cast<int64_t>(k) * NL + a];
    nd[a] = P.nodes[static_cast<int64_t>(k) * NL + a];
#pragma unroll
    for (int d = 0; d < DIM; ++d) X[a][d] = P.coords[static_cast<int64_t>(v) * DIM + d];
  }
  double Bm[DIM][DIM], Bi[DIM][DIM], det;
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) Bm[i][j] = X[j + 1][i] - X[0][i];
  if constexpr (DIM == 2) {
    det = Bm[0][0] * Bm[1][1] - Bm[0][1] * Bm[1][0];
    const double id = 1.0 / det;
    Bi[0][0] = Bm[1][1] * id;  Bi[0][1] = -Bm[0][1] * id;
    Bi[1][0] = -Bm[1][0] * id; Bi[1][1] = Bm[0][0] * id;
  } else {
    const double c00 = Bm[1][1] * Bm[2][2] - Bm[1][2] * Bm[2][1];
    const double c01 = Bm[1][2] * Bm[2][0] - Bm[1][0] * Bm[2][2];
    const double c02 = Bm[1][0] * Bm[2][1] - Bm[1][1] * Bm[2][0];
    det = Bm[0][0] * c00 + Bm[0][1] * c01 + Bm[0][2] * c02;
    const double id = 1.0 / det;
    Bi[0][0] = c00 * id;
    Bi[1][0] = c01 * id;
    Bi[2][0] = c02 * id;
    Bi[0][1] = (Bm[0][2] * Bm[2][1] - Bm[0][1] * Bm[2][2]) * id;
    Bi[1][1] = (Bm[0][0] * Bm[2][2] - Bm[0][2] * Bm[2][0]) * id;
    Bi[2][1] = (Bm[0][1] * Bm[2][0] - Bm[0][0] * Bm[2][1]) * id;
    Bi[0][2] = (Bm[0][1] * Bm[1][2] - Bm[0][2] * Bm[1][1]) * id;
    Bi[1][2] = (Bm[0][2] * Bm[1][0] - Bm[0][0] * Bm[1][2]) * id;
    Bi[2][2] = (Bm[0][0] * Bm[1][1] - Bm[0][1] * Bm[1][0]) * id;
  }
  const double adet = fabs(det);
  const double vol = adet / (DIM == 2 ? 2.0 : 6.0);
  double G[NL][DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    double s = 0.0;
#pragma unroll
    for (int kk = 0; kk < DIM; ++kk) {
      G[kk + 1][j] = Bi[kk][j];
      s += Bi[kk][j];
    }
    G[0][j] = -s;
  }
  const int bs = P.bs, bs2 = bs * bs;
  double c[NL][NS];
#pragma unroll
  for (int a = 0; a < NL; ++a)
#pragma unroll
    for (int s = 0; s < NS; ++s) c[a][s] = P.x[static_cast<int64_t>(nd[a]) * bs + s];
  double R[kMaxDevRegisters];
  double down[NL][NS], up[NL][NS];
  fd_local_residual<DIM, NS>(P, c, X, Bm, G, adet, vol, down, R);
  const int32_t* bp = P.bpos + static_cast<int64_t>(k) * NL * NL;
#pragma unroll 1
  for (int b = 0; b < NL; ++b) {
#pragma unroll 1
    for (int w = 0; w < NS; ++w) {
      double cbw = 0.0;
#pragma unroll
      for (int bb = 0; bb < NL; ++bb)
#pragma unroll
        for (int ww = 0; ww < NS; ++ww)
          if (bb == b && ww == w) cbw = c[bb][ww];
      const double delta = P.fd_eps * (1.0 + fabs(cbw));
      double cp[NL][NS];
#pragma unroll
      for (int bb = 0; bb < NL; ++bb)
#pragma unroll
        for (int ww = 0; ww < NS; ++ww) cp[bb][ww] = (bb == b && ww == w) ? cbw + delta : c[bb][ww];
      fd_local_residual<DIM, NS>(P, cp, X, Bm, G, adet, vol, up, R);
#pragma unroll
      for (int a = 0; a < NL; ++a)
#pragma unroll
        for (int s = 0; s < NS; ++s)
          P.J[static_cast<int64_t>(bp[a * NL + b]) * bs2 + s * bs + w] += (up[a][s] - down[a][s]) / delta;
    }
  }
}

// k_volume with its shared-memory register file and coefficients: 128 threads per block,
// fewer when a large program would need more than kVolumeSmemCap bytes per block
constexpr int kVolumeSmemCap = 160 * 1024;
template <int DIM, int NS, class F>
void launch_volume_kernel(const VolumeParams& p, int begin, int end, int mode, cudaStream_t stream) {
  const int n = end - begin;
  const int64_t per_thread = static_cast<int64_t>(p.prog.nregs + p.ncoef) * static_cast<int64_t>(sizeof(F));
  int threads = 128;
  while (threads > 32 && per_thread * threads > kVolumeSmemCap) threads /= 2;
  const size_t smem = static_cast<size_t>(per_thread * threads);
  // once per instantiation (thread-safe static initialisation)
  static const bool attr_set = [] {
    if (cudaFuncSetAttribute(k_volume<DIM, NS, F>, cudaFuncAttributeMaxDynamicSharedMemorySize, kVolumeSmemCap) !=
        cudaSuccess)
      throw std::runtime_error("k_volume: cannot raise the shared-memory limit");
    return true;
  }();
  (void)attr_set;
  k_volume<DIM, NS, F><<<(n + threads - 1) / threads, threads, smem, stream>>>(p, begin, end, mode);
}

template <int DIM, int NS>
void launch_t(const VolumeParams& p, int begin, int end, int mode, cudaStream_t stream) {
  const int n = end - begin;
  if (n <= 0) return;
  const int threads = 128;
  count_launches(1);
  if (mode == kVolumeNumericalJacobian)
    k_volume_fd<DIM, NS><<<(n + threads - 1) / threads, threads, 0, stream>>>(p, begin, end);
  else if (mode == 2 && p.jac_f32)
    launch_volume_kernel<DIM, NS, float>(p, begin, end, mode, stream);
  else
    launch_volume_kernel<DIM, NS, double>(p, begin, end, mode, stream);
}

}  // namespace

void launch_gather_residual(double* r, int bs, int ns, int64_t node_begin, int64_t nnodes, const int64_t* ptr,
                            const int32_t* list, const double* er, cudaStream_t stream) {
  if (nnodes <= 0 || ns <= 0) return;
  const int64_t total = nnodes * ns;
  if (total >= (int64_t{1} << 32) - 256) throw std::runtime_error("gather: more than 2^32 node entries");
  count_launches(1);
  k_gather_residual<<<static_cast<unsigned>((total + 255) / 256), 256, 0, stream>>>(
      r, bs, static_cast<unsigned>(ns), node_begin, static_cast<unsigned>(total), ptr, list, er);
}

void launch_gather_jacobian(double* J, int bs, int nslot, const int32_t* slot_pos, int64_t block_begin,
                            int64_t nblocks, const int64_t* ptr, const int32_t* list, const double* ej, bool f32,
                            cudaStream_t stream, const JacobianGatherOut& out) {
  if (nblocks <= 0 || nslot <= 0) return;
  const int64_t total = nblocks * nslot;
  if (total >= (int64_t{1} << 32) - 256) throw std::runtime_error("gather: more than 2^32 block entries");
  count_launches(1);
  const unsigned grid = static_cast<unsigned>((total + 255) / 256);
  if (f32)
    k_gather_jacobian<float><<<grid, 256, 0, stream>>>(J, bs * bs, static_cast<unsigned>(nslot), slot_pos, block_begin,
                                                       static_cast<unsigned>(total), ptr, list,
                                                       reinterpret_cast<const float*>(ej), out);
  else
    k_gather_jacobian<double><<<grid, 256, 0, stream>>>(J, bs * bs, static_cast<unsigned>(nslot), slot_pos,
                                                        block_begin, static_cast<unsigned>(total), ptr, list, ej, out);
}

void launch_gather_jacobian_full(double* J, int bs, int nslot, const std::vector<int32_t>& slot_pos_host,
                                 int64_t block_begin, int64_t nblocks, const int64_t* ptr, const int32_t* list,
                                 const double* ej, bool f32, cudaStream_t stream, const JacobianGatherOut& out) {
  if (nblocks <= 0) return;
  const int bs2 = bs * bs;
  if (bs2 > 64) throw std::runtime_error("covering gather: more than 64 entries per block");
  EntrySlots es;
  for (int e = 0; e < 64; ++e) es.slot[e] = -1;
  for (size_t m = 0; m < slot_pos_host.size(); ++m) es.slot[slot_pos_host[m]] = static_cast<int8_t>(m);
  if (nblocks >= (int64_t{1} << 32) - 256) throw std::runtime_error("gather: more than 2^32 blocks");
  const unsigned nb = static_cast<unsigned>(nblocks);
  const unsigned bgrid = (nb + kBlockGatherThreads - 1) / kBlockGatherThreads;
#define DC_BLOCKS(B2)                                                                                           \
  if (bs2 == B2) {                                                                                              \
    count_launches(1);                                                                                          \
    if (f32)                                                                                                    \
      k_gather_jacobian_blocks<float, B2><<<bgrid, kBlockGatherThreads, 0, stream>>>(                           \
          J, nslot, es, block_begin, nb, ptr, list, reinterpret_cast<const float*>(ej), out);                   \
    else                                                                                                        \
      k_gather_jacobian_blocks<double, B2><<<bgrid, kBlockGatherThreads, 0, stream>>>(J, nslot, es, block_begin, \
                                                                                       nb, ptr, list, ej, out); \
    return;                                                                                                     \
  }
  DC_BLOCKS(1) DC_BLOCKS(4) DC_BLOCKS(9) DC_BLOCKS(16) DC_BLOCKS(25)
#undef DC_BLOCKS
  const int64_t total = nblocks * bs2;
  if (total >= (int64_t{1} << 32) - 256) throw std::runtime_error("gather: more than 2^32 block entries");
  count_launches(1);
  const unsigned grid = static_cast<unsigned>((total + 255) / 256);
  if (f32)
    k_gather_jacobian_full<float><<<grid, 256, 0, stream>>>(J, bs2, static_cast<unsigned>(nslot), es, block_begin,
                                                            static_cast<unsigned>(total), ptr, list,
                                                            reinterpret_cast<const float*>(ej), out);
  else
    k_gather_jacobian_full<double><<<grid, 256, 0, stream>>>(J, bs2, static_cast<unsigned>(nslot), es, block_begin,
                                                             static_cast<unsigned>(total), ptr, list, ej, out);
}

void launch_volume(int dim, int ns, const VolumeParams& p, int begin, int end, int mode,
                   cudaStream_t stream) {
#define DC_CASE(D, S) \
  if (dim == D && ns == S) return launch_t<D, S>(p, begin, end, mode, stream);
  DC_CASE(2, 1) DC_CASE(2, 2) DC_CASE(2, 3) DC_CASE(2, 4) DC_CASE(2, 5) DC_CASE(2, 6) DC_CASE(2, 7) DC_CASE(2, 8)
  DC_CASE(3, 1) DC_CASE(3, 2) DC_CASE(3, 3) DC_CASE(3, 4) DC_CASE(3, 5) DC_CASE(3, 6) DC_CASE(3, 7) DC_CASE(3, 8)
#undef DC_CASE
  throw std::runtime_error("volume assembly supports dimension 2/3 and 1..8 species per compartment, got dim=" +
                           std::to_string(dim) + " species=" + std::to_string(ns));
}

}  // namespace dcgpu
