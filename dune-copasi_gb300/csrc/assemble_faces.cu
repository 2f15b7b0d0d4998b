// Interface / boundary outflow assembly (local_operator.hh:777-971 residual,
// :973-1203 analytic Jacobian, :1398-1436 boundary).
//
// One thread per face of one colour class.  On a conforming P1 face the basis functions
// of both neighbouring cells restrict to the face barycentric coordinates, so the
// coefficients of the face vertices of each side's compartment give the values at the
// face quadrature points; gradients (only loaded when a program reads them) come from
// the full neighbouring cells.  Values of species living on the other side are taken at
// the same physical point through the other side's own cell.
#include <algorithm>
#include <stdexcept>

#include "assemble.cuh"
#include "interp.cuh"
#include "linalg.cuh"

namespace dcgpu {

namespace {

constexpr int kFaceMaxSpecies = 8;

template <int DIM> struct FaceRule;
template <> struct FaceRule<2> {
  static constexpr int NQ = 2;
  __device__ static double lam(int q, int k) {
    const double s = (q == 0) ? 0.5 - 0.28867513459481288225 : 0.5 + 0.28867513459481288225;
    return k == 0 ? 1.0 - s : s;
  }
  __device__ static constexpr double w(int) { return 0.5; }
};
template <> struct FaceRule<3> {
  static constexpr int NQ = 3;
  __device__ static double lam(int q, int k) {
    const double x0 = (q == 0) ? 2.0 / 3.0 : 1.0 / 6.0;
    const double x1 = (q == 1) ? 2.0 / 3.0 : 1.0 / 6.0;
    return k == 0 ? 1.0 - x0 - x1 : (k == 1 ? x0 : x1);
  }
  __device__ static constexpr double w(int) { return 1.0 / 6.0; }
};

// gradient of the species of one side inside cell e (P1, affine)
template <int DIM>
__device__ void cell_gradients(const FaceParams& P, int side, int e, int ns, double (*grad)[3]) {
  constexpr int NL = DIM + 1;
  double X[NL][DIM];
  int nd[NL];
  for (int a = 0; a < NL; ++a) {
    const int v = P.cells[static_cast<int64_t>(e) * NL + a];
    nd[a] = P.vnode[side][v];
    for (int d = 0; d < DIM; ++d) X[a][d] = P.coords[static_cast<int64_t>(v) * DIM + d];
  }
  double Bm[DIM][DIM], Bi[DIM][DIM];
  for (int i = 0; i < DIM; ++i)
    for (int j = 0; j < DIM; ++j) Bm[i][j] = X[j + 1][i] - X[0][i];
  if constexpr (DIM == 2) {
    const double det = Bm[0][0] * Bm[1][1] - Bm[0][1] * Bm[1][0];
    Bi[0][0] = Bm[1][1] / det;  Bi[0][1] = -Bm[0][1] / det;
    Bi[1][0] = -Bm[1][0] / det; Bi[1][1] = Bm[0][0] / det;
  } else {
    const double c00 = Bm[1][1] * Bm[2][2] - Bm[1][2] * Bm[2][1];
    const double c01 = Bm[1][2] * Bm[2][0] - Bm[1][0] * Bm[2][2];
    const double c02 = Bm[1][0] * Bm[2][1] - Bm[1][1] * Bm[2][0];
    const double det = Bm[0][0] * c00 + Bm[0][1] * c01 + Bm[0][2] * c02;
    Bi[0][0] = c00 / det; Bi[1][0] = c01 / det; Bi[2][0] = c02 / det;
    Bi[0][1] = (Bm[0][2] * Bm[2][1] - Bm[0][1] * Bm[2][2]) / det;
    Bi[1][1] = (Bm[0][0] * Bm[2][2] - Bm[0][2] * Bm[2][0]) / det;
    Bi[2][1] = (Bm[0][1] * Bm[2][0] - Bm[0][0] * Bm[2][1]) / det;
    Bi[0][2] = (Bm[0][1] * Bm[1][2] - Bm[0][2] * Bm[1][1]) / det;
    Bi[1][2] = (Bm[0][2] * Bm[1][0] - Bm[0][0] * Bm[1][2]) / det;
    Bi[2][2] = (Bm[0][0] * Bm[1][1] - Bm[0][1] * Bm[1][0]) / det;
  }
  double G[NL][DIM];
  for (int j = 0; j < DIM; ++j) {
    double s = 0.0;
    for (int k = 0; k < DIM; ++k) { G[k + 1][j] = Bi[k][j]; s += Bi[k][j]; }
    G[0][j] = -s;
  }
  for (int s = 0; s < ns; ++s)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      if (j < DIM)
        for (int a = 0; a < NL; ++a)
          acc += P.x[static_cast<int64_t>(nd[a]) * P.bs + s] * G[a][j];
      grad[s][j] = acc;
    }
}

// The outflow terms of side `side` of face f at the face-vertex coefficients cf of both sides:
// residual contributions rl[k][s] (face vertex k, species s of the side's compartment) when
// do_res, and the analytic Jacobian coefficients of the side's terms when coef is non-null.
// Gradients (read only when a program asks for one) come from the cells' own coefficients.
template <int DIM>
__device__ void face_side(const FaceParams& P, int f, int side, bool has_out,
                          const double (&cf)[2][DIM][kFaceMaxSpecies], const double (&Xf)[DIM][DIM],
                          const double (&nrm)[DIM], double ielem, double fvol, bool do_res,
                          double (&rl)[DIM][kFaceMaxSpecies], double* coef, double* R) {
  constexpr int NF = DIM;
  constexpr int NQ = FaceRule<DIM>::NQ;
  const int other = 1 - side;
  bool need_grad = false;
  for (int i = 0; i < P.prog[side].ninputs; ++i) {
    const uint16_t id = P.prog[side].inputs[i];
    need_grad |= (id >= IN_GRAD && id < IN_POSITION);
  }
  double grad[2][kFaceMaxSpecies][3];
  for (int sd = 0; sd < 2; ++sd)
    for (int s = 0; s < kFaceMaxSpecies; ++s)
      for (int j = 0; j < 3; ++j) grad[sd][s][j] = 0.0;
  if (need_grad) {
    const int e_side = side == 0 ? P.elem_in[f] : P.elem_out[f];
    const int e_other = side == 0 ? P.elem_out[f] : P.elem_in[f];
    if (P.ns[side] > 0) cell_gradients<DIM>(P, side, e_side, P.ns[side], grad[side]);
    if (has_out && P.ns[other] > 0) cell_gradients<DIM>(P, other, e_other, P.ns[other], grad[other]);
  }
  const double sgn = side == 0 ? 1.0 : -1.0;
  for (int k = 0; k < NF; ++k)
    for (int s = 0; s < kFaceMaxSpecies; ++s) rl[k][s] = 0.0;
  const int nt = P.n_terms[side];
  const Term* terms = P.terms[side];
  for (int q = 0; q < NQ; ++q) {
    double lam[NF];
    for (int k = 0; k < NF; ++k) lam[k] = FaceRule<DIM>::lam(q, k);
    double xq[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < DIM; ++d)
      for (int k = 0; k < NF; ++k) xq[d] += lam[k] * Xf[k][d];
    const double fq = FaceRule<DIM>::w(q) * ielem;
    for (int i = 0; i < P.prog[side].ninputs; ++i) {
      const uint16_t id = P.prog[side].inputs[i];
      double v = 0.0;
      if (id < IN_GRAD || (id >= IN_GRAD && id < IN_POSITION)) {
        const bool is_grad = id >= IN_GRAD;
        const int gi = is_grad ? (id - IN_GRAD) / 3 : id;
        const int ax = is_grad ? (id - IN_GRAD) % 3 : 0;
        for (int sd = 0; sd < 2; ++sd) {
          const int ls = gi - P.species_offset[sd];
          if (ls >= 0 && ls < P.ns[sd] && (sd == 0 || has_out)) {
            if (is_grad) {
              v = grad[sd][ls][ax];
            } else {
              double acc = 0.0;
              for (int k = 0; k < NF; ++k) acc += cf[sd][k][ls] * lam[k];
              v = acc;
            }
          }
        }
      } else if (id < IN_NORMAL) {
        v = xq[id - IN_POSITION];
      } else if (id < IN_TIME) {
        const int ax = id - IN_NORMAL;
        v = ax < DIM ? sgn * nrm[ax] : 0.0;
      } else if (id == IN_TIME) {
        v = P.t;
      } else if (id == IN_ENTITY_VOLUME) {
        v = fvol;
      } else if (id == IN_IN_BOUNDARY) {
        v = has_out ? 0.0 : 1.0;
      } else if (id == IN_IN_SKELETON) {
        v = has_out ? 1.0 : 0.0;
      }
      R[i] = v;
    }
    run_program<double>(P.prog[side], P.tables, R);
    const uint8_t* out = P.prog[side].outputs;
    for (int t = 0; t < nt; ++t) {
      const Term T = terms[t];
      const double o = R[out[T.out]] * P.ca * fq;
      if (T.kind == F_OUTFLOW) {
        if (do_res)
          for (int k = 0; k < NF; ++k) rl[k][T.test] += o * lam[k];
      } else if (T.kind == F_OUTFLOW_JAC) {
        if (coef) coef[T.coef + q] = o;
      }
    }
  }
}

// face vertices, their block rows on both sides, coordinates and coefficients
template <int DIM>
__device__ void face_load(const FaceParams& P, int f, int (&node)[2][DIM], double (&Xf)[DIM][DIM],
                          double (&cf)[2][DIM][kFaceMaxSpecies]) {
  constexpr int NF = DIM;
  for (int k = 0; k < NF; ++k) {
    const int fv = P.fverts[static_cast<int64_t>(f) * NF + k];
    node[0][k] = P.node_in[static_cast<int64_t>(f) * NF + k];
    node[1][k] = P.node_out[static_cast<int64_t>(f) * NF + k];
    for (int d = 0; d < DIM; ++d) Xf[k][d] = P.coords[static_cast<int64_t>(fv) * DIM + d];
  }
  for (int sd = 0; sd < 2; ++sd)
    for (int k = 0; k < NF; ++k)
      for (int s = 0; s < kFaceMaxSpecies; ++s)
        cf[sd][k][s] = (s < P.ns[sd] && node[sd][k] >= 0)
                           ? P.x[static_cast<int64_t>(node[sd][k]) * P.bs + s] : 0.0;
}

template <int DIM>
__global__ void __launch_bounds__(128) k_faces(const FaceParams P, const int begin, const int end,
                                               const int mode) {
  constexpr int NF = DIM;
  constexpr int NQ = FaceRule<DIM>::NQ;
  const int f = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= end) return;
  const bool has_out = P.elem_out[f] >= 0;
  const int bs = P.bs, bs2 = bs * bs;
  int node[2][NF];
  double Xf[NF][DIM], cf[2][NF][kFaceMaxSpecies];
  face_load<DIM>(P, f, node, Xf, cf);
  double nrm[DIM];
  for (int d = 0; d < DIM; ++d) nrm[d] = P.normal[static_cast<int64_t>(f) * DIM + d];
  const double ielem = P.ielem[f];
  const double fvol = P.fvolume[f];
  const bool do_res = (mode & 1) && P.r;
  const bool do_apply = (mode & kFaceJacobianApply) != 0;  // matrix-free: y += J_face v
  const bool do_jac = ((mode & 2) && P.J) || do_apply;

  double R[kMaxDevRegisters];
  for (int side = 0; side < 2; ++side) {
    if (P.n_terms[side] == 0) continue;
    if (side == 1 && !has_out) continue;
    const int other = 1 - side;
    double rl[NF][kFaceMaxSpecies];
    double coef[kMaxCoefficients];
    face_side<DIM>(P, f, side, has_out, cf, Xf, nrm, ielem, fvol, do_res, rl, do_jac ? coef : nullptr, R);
    if (do_res)
      for (int k = 0; k < NF; ++k)
        for (int s = 0; s < P.ns[side]; ++s)
          P.r[static_cast<int64_t>(node[side][k]) * bs + s] += rl[k][s];
    if (do_jac) {
      const int nt = P.n_terms[side];
      const Term* terms = P.terms[side];
      for (int t = 0; t < nt; ++t) {
        const Term T = terms[t];
        if (T.kind != F_OUTFLOW_JAC) continue;
        const int col_side = T.side ? other : side;
        const int pair = side * 2 + col_side;
        const int32_t* bp = P.bpos + (static_cast<int64_t>(f) * 4 + pair) * NF * NF;
        for (int k = 0; k < NF; ++k)
          for (int l = 0; l < NF; ++l) {
            double v = 0.0;
            for (int q = 0; q < NQ; ++q)
              v += coef[T.coef + q] * FaceRule<DIM>::lam(q, k) * FaceRule<DIM>::lam(q, l);
            if (do_apply)
              P.y[static_cast<int64_t>(node[side][k]) * bs + T.test] +=
                  v * P.v[static_cast<int64_t>(node[col_side][l]) * bs + T.trial];
            else
              P.J[static_cast<int64_t>(bp[k * NF + l]) * bs2 + T.test * bs + T.trial] += v;
          }
      }
    }
  }
}

// Numerical Jacobian of the outflow terms (local_operator.hh:1205-1344): every face-vertex
// coefficient of the first side, then of the second, is moved by delta = eps (1 + |c|) and the
// change of both sides' face residuals divided by it.  Only face-vertex coefficients enter the
// face residual when no program reads a gradient (the model rejects the numerical Jacobian
// otherwise), so the other cell coefficients' columns are zero.
template <int DIM>
__global__ void __launch_bounds__(128) k_faces_fd(const FaceParams P, const int begin, const int end, double eps) {
  constexpr int NF = DIM;
  const int f = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= end) return;
  const bool has_out = P.elem_out[f] >= 0;
  const int bs = P.bs, bs2 = bs * bs;
  int node[2][NF];
  double Xf[NF][DIM], cf[2][NF][kFaceMaxSpecies];
  face_load<DIM>(P, f, node, Xf, cf);
  double nrm[DIM];
  for (int d = 0; d < DIM; ++d) nrm[d] = P.normal[static_cast<int64_t>(f) * DIM + d];
  const double ielem = P.ielem[f];
  const double fvol = P.fvolume[f];
  double R[kMaxDevRegisters];
  double down[2][NF][kFaceMaxSpecies], up[NF][kFaceMaxSpecies];
  bool active[2];
  for (int side = 0; side < 2; ++side) {
    active[side] = P.n_terms[side] > 0 && (side == 0 || has_out);
    if (active[side]) face_side<DIM>(P, f, side, has_out, cf, Xf, nrm, ielem, fvol, true, down[side], nullptr, R);
  }
  for (int sigma = 0; sigma < 2; ++sigma) {
    if (sigma == 1 && !has_out) continue;
    for (int l = 0; l < NF; ++l) {
      if (node[sigma][l] < 0) continue;
      for (int w = 0; w < P.ns[sigma]; ++w) {
        const double c0 = cf[sigma][l][w];
        const double delta = eps * (1.0 + fabs(c0));
        cf[sigma][l][w] = c0 + delta;
        for (int rho = 0; rho < 2; ++rho) {
          if (!active[rho]) continue;
          face_side<DIM>(P, f, rho, has_out, cf, Xf, nrm, ielem, fvol, true, up, nullptr, R);
          const int32_t* bp = P.bpos + (static_cast<int64_t>(f) * 4 + rho * 2 + sigma) * NF * NF;
          for (int k = 0; k < NF; ++k) {
            if (node[rho][k] < 0) continue;
            const int32_t blk = bp[k * NF + l];
            if (blk < 0) continue;
            for (int s = 0; s < P.ns[rho]; ++s)
              P.J[static_cast<int64_t>(blk) * bs2 + s * bs + w] += (up[k][s] - down[rho][k][s]) / delta;
          }
        }
        cf[sigma][l][w] = c0;
      }
    }
  }
}

__global__ void k_pad_identity(const int32_t* diag, const int8_t* row_ns, int nrows, int bs, double* J,
                               double value) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows) return;
  const int64_t base = static_cast<int64_t>(diag[i]) * bs * bs;
  for (int s = row_ns[i]; s < bs; ++s) J[base + s * bs + s] += value;
}

// constrained entries (blocked index idx[k]): op 0 sets v[idx] = val, op 1 zeroes v[idx]
__global__ void k_constraints(double* v, const int64_t* __restrict__ idx, const double* __restrict__ val, int64_t n,
                              int op) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  v[idx[k]] = op == 0 ? val[k] : 0.0;
}

// constrained Jacobian rows become unit rows: a thread per constraint clears scalar row i
// of block row br in every block of the row and puts 1 on the diagonal.  Constraints in
// one block row have different i, so no two threads write the same entry.
__global__ void k_constraint_rows(double* J, ConstraintRows cr, const int64_t* __restrict__ idx, int64_t n, int bs) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t br = idx[k] / bs;
  const int i = static_cast<int>(idx[k] % bs);
  const int64_t bs2 = static_cast<int64_t>(bs) * bs;
  for (int32_t b = cr.rowptr[br]; b < cr.rowptr[br + 1]; ++b)
    for (int j = 0; j < bs; ++j) J[b * bs2 + i * bs + j] = 0.0;
  J[static_cast<int64_t>(cr.diag[br]) * bs2 + i * bs + i] = 1.0;
}

// y = v on the rows whose Jacobian row is a unit row: padded species slots (row_ns[i] <= s
// < bs) and constrained DOFs
__global__ void k_unit_rows_apply(const int8_t* __restrict__ row_ns, int64_t nrows, int bs, const int64_t* __restrict__ cons,
                                  int64_t ncons, const double* __restrict__ v, double* __restrict__ y) {
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (row_ns && t < nrows)
    for (int s = row_ns[t]; s < bs; ++s) y[t * bs + s] = v[t * bs + s];
  if (t < ncons) y[cons[t]] = v[cons[t]];
}

}  // namespace

void launch_unit_rows_apply(const int8_t* row_ns, int64_t nrows, int bs, const int64_t* cons, int64_t ncons,
                            const double* v, double* y, cudaStream_t stream) {
  const int64_t n = std::max<int64_t>(row_ns ? nrows : 0, ncons);
  if (n <= 0) return;
  count_launches(1);
  k_unit_rows_apply<<<static_cast<int>((n + 255) / 256), 256, 0, stream>>>(row_ns, nrows, bs, cons, ncons, v, y);
}

void launch_constraints(double* v, const int64_t* idx, const double* val, int64_t n, int op, cudaStream_t stream) {
  if (n <= 0) return;
  count_launches(1);
  k_constraints<<<static_cast<int>((n + 255) / 256), 256, 0, stream>>>(v, idx, val, n, op);
}

void launch_constraint_rows(double* J, const ConstraintRows& cr, const int64_t* idx, int64_t n, int bs,
                            cudaStream_t stream) {
  if (n <= 0) return;
  count_launches(1);
  k_constraint_rows<<<static_cast<int>((n + 127) / 128), 128, 0, stream>>>(J, cr, idx, n, bs);
}

void launch_faces(int dim, const FaceParams& p, int begin, int end, int mode, cudaStream_t stream) {
  const int n = end - begin;
  if (n <= 0) return;
  const int threads = 128;
  const int blocks = (n + threads - 1) / threads;
  count_launches(1);
  if (dim == 2) k_faces<2><<<blocks, threads, 0, stream>>>(p, begin, end, mode);
  else if (dim == 3) k_faces<3><<<blocks, threads, 0, stream>>>(p, begin, end, mode);
  else throw std::runtime_error("faces: unsupported dimension");
}

void launch_faces_fd(int dim, const FaceParams& p, int begin, int end, double eps, cudaStream_t stream) {
  const int n = end - begin;
  if (n <= 0) return;
  const int threads = 128;
  const int blocks = (n + threads - 1) / threads;
  count_launches(1);
  if (dim == 2) k_faces_fd<2><<<blocks, threads, 0, stream>>>(p, begin, end, eps);
  else if (dim == 3) k_faces_fd<3><<<blocks, threads, 0, stream>>>(p, begin, end, eps);
  else throw std::runtime_error("faces: unsupported dimension");
}

void launch_pad_identity(const int32_t* diag, const int8_t* row_ns, int nrows, int bs, double* J,
                         double value, cudaStream_t stream) {
  if (nrows <= 0) return;
  count_launches(1);
  k_pad_identity<<<(nrows + 255) / 256, 256, 0, stream>>>(diag, row_ns, nrows, bs, J, value);
}

}  // namespace dcgpu
