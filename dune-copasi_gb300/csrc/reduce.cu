// Device side of the transform/reduce operators
// (dune/copasi/model/diffusion_reaction/reduce.hh:40-285): the evaluation expressions of
// all keys at every point of the order-4 rule of every cell, and the sum / max / min folds.
#include <cfloat>
#include <stdexcept>

#include "interp.cuh"
#include "linalg.cuh"
#include "reduce.cuh"

namespace dcgpu {

namespace {

// order-4 rules of the reduce operators, by barycentric coordinates (lambda_0..lambda_d):
// triangles, two (a, a, 1-2a) orbits (exact to degree 4); tetrahedra, two (a, a, a, 1-3a)
// orbits and one (b, b, 1/2-b, 1/2-b) orbit (exact to degree 5).  Orbit parameters solve
// the moment equations; the CPU oracle lists the same points in the same order.
template <int DIM> struct ReduceRule;
template <> struct ReduceRule<2> {
  static constexpr int NQ = 6;
  __device__ static double lam(int q, int k) {
    const double a = q < 3 ? 0.4459484909159645 : 0.09157621350977077;
    const int r = q % 3;  // position of the 1-2a entry: 2, 1, 0
    return k == 2 - r ? 1.0 - 2.0 * a : a;
  }
  __device__ static double w(int q) { return q < 3 ? 0.11169079483900554 : 0.05497587182766112; }
};
template <> struct ReduceRule<3> {
  static constexpr int NQ = 14;
  __device__ static double lam(int q, int k) {
    if (q < 8) {
      const double a = q < 4 ? 0.0927352503108912 : 0.3108859192633006;
      const int r = q % 4;  // position of the 1-3a entry: 3, 2, 1, 0
      return k == 3 - r ? 1.0 - 3.0 * a : a;
    }
    const double b = 0.0455037041256496, c = 0.5 - b;
    // (b,b,c,c) (b,c,b,c) (b,c,c,b) (c,b,b,c) (c,b,c,b) (c,c,b,b)
    const int pat[6] = {0x3, 0x5, 0x6, 0x9, 0xA, 0xC};  // bit k set: entry k is c
    return (pat[q - 8] >> (3 - k)) & 1 ? c : b;
  }
  __device__ static double w(int q) {
    return q < 4 ? 0.01224884051939366 : q < 8 ? 0.01878132095300264 : 0.007091003462846911;
  }
};

template <int DIM>
__global__ void __launch_bounds__(128) k_reduce_eval(const ReduceParams P) {
  constexpr int NL = DIM + 1;
  constexpr int NQ = ReduceRule<DIM>::NQ;
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  double X[NL][DIM];
  int nd[NL];
#pragma unroll
  for (int a = 0; a < NL; ++a) {
    const int v = P.cells[e * NL + a];
    nd[a] = P.cell_nodes[e * NL + a];
#pragma unroll
    for (int d = 0; d < DIM; ++d) X[a][d] = P.coords[static_cast<int64_t>(v) * DIM + d];
  }
  const int comp = P.cell_comp[e];
  double Bm[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) Bm[i][j] = X[j + 1][i] - X[0][i];
  double det, Bi[DIM][DIM];
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
  double G[NL][DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      G[k + 1][j] = Bi[k][j];
      s += Bi[k][j];
    }
    G[0][j] = -s;
  }
  double R[kMaxDevRegisters];
  const int64_t npts = P.ne * NQ;
#pragma unroll 1
  for (int q = 0; q < NQ; ++q) {
    double lam[NL], xq[DIM];
#pragma unroll
    for (int a = 0; a < NL; ++a) lam[a] = ReduceRule<DIM>::lam(q, a);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      double acc = 0.0;
#pragma unroll
      for (int a = 0; a < NL; ++a) acc += lam[a] * X[a][d];
      xq[d] = acc;
    }
    for (int i = 0; i < P.prog.ninputs; ++i) {
      const uint16_t id = P.prog.inputs[i];
      double v = 0.0;
      if (id < IN_POSITION) {
        // species value or gradient component: zero unless the species' compartment holds the cell
        const bool grad = id >= IN_GRAD;
        const int gi = grad ? (id - IN_GRAD) / 3 : id;
        const int ax = grad ? (id - IN_GRAD) % 3 : 0;
        if (comp >= 0 && P.sp_comp[gi] == comp && nd[0] >= 0) {
          const int loc = P.sp_local[gi];
#pragma unroll
          for (int a = 0; a < NL; ++a) {
            const double c = P.x[static_cast<int64_t>(nd[a]) * P.bs + loc];
            if (grad) {
#pragma unroll
              for (int d = 0; d < DIM; ++d)
                if (d == ax) v += c * G[a][d];
            } else {
              v += c * lam[a];
            }
          }
        }
      } else if (id < IN_NORMAL) {
#pragma unroll
        for (int d = 0; d < DIM; ++d)
          if (d == id - IN_POSITION) v = xq[d];
      } else if (id == IN_TIME) {
        v = P.t;
      } else if (id == IN_ENTITY_VOLUME) {
        v = adet / (DIM == 2 ? 2.0 : 6.0);
      } else if (id == IN_INTEGRATION_FACTOR) {
        v = ReduceRule<DIM>::w(q) * adet;
      } else if (id == IN_IN_VOLUME) {
        v = 1.0;
      }
      R[i] = v;
    }
    run_program<double>(P.prog, P.tables, R);
    for (int k = 0; k < P.nkeys; ++k) P.out[k * npts + e * NQ + q] = R[P.prog.outputs[k]];
  }
}

constexpr int kFoldThreads = 256;

// op 0: sum, 1: max, 2: min; deterministic: per-block partials added by the last block in
// block order
__global__ void __launch_bounds__(kFoldThreads) k_fold(const double* __restrict__ v, int64_t n, int op,
                                                       double* partial, unsigned* counter, double* out) {
  __shared__ double sh[kFoldThreads];
  __shared__ bool last;
  const double ident = op == 0 ? 0.0 : (op == 1 ? -DBL_MAX : DBL_MAX);
  auto comb = [op](double a, double b) { return op == 0 ? a + b : (op == 1 ? fmax(a, b) : fmin(a, b)); };
  double acc = ident;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    acc = comb(acc, v[i]);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kFoldThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = comb(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = sh[0];
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double r = ident;
  for (unsigned b = 0; b < gridDim.x; ++b) r = comb(r, __ldcg(&partial[b]));
  *out = r;
  *counter = 0u;
}

}  // namespace

int reduce_points(int dim) { return dim == 2 ? ReduceRule<2>::NQ : ReduceRule<3>::NQ; }

void launch_reduce_eval(int dim, const ReduceParams& p, cudaStream_t s) {
  if (p.ne == 0) return;
  const int threads = 128;
  const int blocks = static_cast<int>((p.ne + threads - 1) / threads);
  count_launches(1);
  if (dim == 2) k_reduce_eval<2><<<blocks, threads, 0, s>>>(p);
  else if (dim == 3) k_reduce_eval<3><<<blocks, threads, 0, s>>>(p);
  else throw std::runtime_error("reduce: unsupported dimension");
}

void launch_fold(const double* v, int64_t n, int op, double* partial, int nblocks, unsigned* counter, double* out,
                 cudaStream_t s) {
  count_launches(1);
  k_fold<<<nblocks, kFoldThreads, 0, s>>>(v, n, op, partial, counter, out);
}

}  // namespace dcgpu
