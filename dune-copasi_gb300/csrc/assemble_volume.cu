// Volume assembly kernels: residual and analytic Jacobian of the mass and stiffness
// forms (dune/copasi/model/diffusion_reaction/local_operator.hh:417-491, 541-707).
#include <cstdio>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "assemble.cuh"
#include "interp.cuh"
#include "linalg.cuh"

namespace dcgpu {

namespace {

// order-2 simplex rules (the same tables as the CPU oracle)
template <int DIM> struct Rule;
template <> struct Rule<2> {
  static constexpr int NQ = 3;
  __host__ __device__ static constexpr double xi(int q, int k) {
    return (q == 0) ? (k == 0 ? 2.0 / 3.0 : 1.0 / 6.0)
         : (q == 1) ? (k == 0 ? 1.0 / 6.0 : 2.0 / 3.0)
                    : 1.0 / 6.0;
  }
  __host__ __device__ static constexpr double w(int) { return 1.0 / 6.0; }
};
template <> struct Rule<3> {
  static constexpr int NQ = 4;
  __host__ __device__ static constexpr double xi(int q, int k) {
    // q = 0: (b,b,b); q = 1..3: a in coordinate q-1
    return (q == k + 1) ? 0.5854101966249685 : 0.1381966011250105;
  }
  __host__ __device__ static constexpr double w(int) { return 1.0 / 24.0; }
};

template <int DIM> struct MassConst;

// P1 basis function a at point q: 1 - (xi_0 + ... ) for a = 0 and xi_{a-1} otherwise, the
// sum formed left to right as the oracle's numpy sum does, so the partition of unity has the
// same bits on both sides (a table of a step function of the state, evaluated at a
// quadrature point on a step, then picks the same step).  The point loop is not unrolled,
// so the values come from constant tables formed at compile time rather than from FP64
// arithmetic per point.
template <int DIM>
__host__ __device__ constexpr double phi_value(int q, int a) {
  if (a > 0) return Rule<DIM>::xi(q, a - 1);
  double s = 0.0;
  for (int k = 0; k < DIM; ++k) s += Rule<DIM>::xi(q, k);
  return 1.0 - s;
}
template <int DIM, class F>
struct PhiTable {
  F v[Rule<DIM>::NQ][DIM + 1];
};
template <int DIM, class F>
constexpr PhiTable<DIM, F> make_phi_table() {
  PhiTable<DIM, F> t{};
  for (int q = 0; q < Rule<DIM>::NQ; ++q)
    for (int a = 0; a <= DIM; ++a) t.v[q][a] = static_cast<F>(phi_value<DIM>(q, a));
  return t;
}
__constant__ PhiTable<2, double> c_phi2d = make_phi_table<2, double>();
__constant__ PhiTable<3, double> c_phi3d = make_phi_table<3, double>();
__constant__ PhiTable<2, float> c_phi2f = make_phi_table<2, float>();
__constant__ PhiTable<3, float> c_phi3f = make_phi_table<3, float>();

template <int DIM, class F>
__device__ __forceinline__ F phi_t(int q, int a) {
  if constexpr (std::is_same_v<F, double>) return DIM == 2 ? c_phi2d.v[q][a] : c_phi3d.v[q][a];
  else return DIM == 2 ? c_phi2f.v[q][a] : c_phi3f.v[q][a];
}
template <int DIM>
__device__ __forceinline__ double phi(int q, int a) {
  return phi_t<DIM, double>(q, a);
}
// reference coordinate k of point q in the arithmetic type F
template <int DIM, class F>
__device__ __forceinline__ F xi_t(int q, int k) {
  constexpr F al = static_cast<F>(MassConst<DIM>::alpha), be = static_cast<F>(MassConst<DIM>::beta);
  // the point's vertex in 0..DIM; reference coordinate k belongs to vertex k + 1
  const int vq = DIM == 2 ? (q == 2 ? 0 : q + 1) : q;
  return vq == k + 1 ? al : be;
}

// Both rules have one point per vertex: point q carries the large barycentric weight
// alpha at vertex vertex_of<DIM>(q) and beta elsewhere, so phi_a(q) phi_b(q) =
// beta^2 + beta (alpha - beta) ([a = v(q)] + [b = v(q)]) + (alpha - beta)^2 [a = b = v(q)].
// A mass-type element matrix sum_q c_q phi_a(q) phi_b(q) is then
// beta^2 S + k1 (c_a + c_b) + [a = b] k2 c_a with S = sum_q c_q and c_a the weight of the
// point at vertex a: two additions per entry instead of NQ multiply-adds.
template <int DIM>
__device__ __forceinline__ constexpr int point_of_vertex(int a) {
  // 2D: points 0, 1, 2 sit at vertices 1, 2, 0; 3D: point q at vertex q
  return DIM == 2 ? (a == 0 ? 2 : a - 1) : a;
}
template <int DIM> struct MassConst;
template <> struct MassConst<2> {
  static constexpr double alpha = 2.0 / 3.0, beta = 1.0 / 6.0;
};
template <> struct MassConst<3> {
  static constexpr double alpha = 0.5854101966249685, beta = 0.1381966011250105;
};

template <int DIM, int NS, class F = double>
__device__ __forceinline__ F volume_input(uint16_t id, const F (&u)[NS], const F (&g)[NS][DIM], const F (&xq)[DIM],
                                          F t, F vol, int soff) {
  if (id < IN_GRAD) {
    const int s = static_cast<int>(id) - soff;
    F v = F(0);
#pragma unroll
    for (int i = 0; i < NS; ++i)
      if (i == s) v = u[i];
    return v;
  }
  if (id < IN_POSITION) {
    const int gi = static_cast<int>(id) - IN_GRAD;
    const int s = gi / 3 - soff, ax = gi % 3;
    F v = F(0);
#pragma unroll
    for (int i = 0; i < NS; ++i)
#pragma unroll
      for (int d = 0; d < DIM; ++d)
        if (i == s && d == ax) v = g[i][d];
    return v;
  }
  if (id < IN_NORMAL) {
    const int ax = static_cast<int>(id) - IN_POSITION;
    F v = F(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d)
      if (d == ax) v = xq[d];
    return v;
  }
  switch (id) {
    case IN_TIME: return t;
    case IN_ENTITY_VOLUME: return vol;
    case IN_IN_VOLUME: return F(1);
    default: return F(0);
  }
}

// Element Jacobian slot values from the per-term coefficients: for every local pair (a, b)
// the terms (sorted by slot) are summed per slot and each slot stored once.  With only
// mass-type terms the element matrix is symmetric and only a <= b is evaluated.  JT is the
// arithmetic and storage type (fp64, or fp32 for the mixed-precision path).
template <int DIM, class JT, class Coef>
__device__ __forceinline__ void element_jacobian(const VolumeParams& P, Coef coef, const JT (&G)[DIM + 1][DIM],
                                                 JT* ej) {
  constexpr int NL = DIM + 1;
  constexpr int NQ = Rule<DIM>::NQ;
  constexpr double al = MassConst<DIM>::alpha, be = MassConst<DIM>::beta;
  const JT k1 = static_cast<JT>(be * (al - be)), k2 = static_cast<JT>((al - be) * (al - be));
  const int nslot = P.n_slots;
#pragma unroll
  for (int a = 0; a < NL; ++a) {
#pragma unroll
    for (int b = 0; b < NL; ++b) {
      if (P.all_mass && b < a) continue;
      int cur = -1;
      JT acc = JT(0);
      for (int t = 0; t < P.n_jac_terms; ++t) {
        const Term T = P.jac_terms[t];
        JT v = JT(0);
        switch (T.kind) {
          case J_MASS:
          case J_MASS_U:
          case J_STORAGE_SELF: {
            const JT ca = coef[T.coef + point_of_vertex<DIM>(a)];
            v = coef[T.coef + NQ] + k1 * (ca + coef[T.coef + point_of_vertex<DIM>(b)]);
            if (a == b) v += k2 * ca;
            break;
          }
          case J_DIFF_SCALAR: {
            JT gg = JT(0);
#pragma unroll
            for (int j = 0; j < DIM; ++j) gg += G[a][j] * G[b][j];
            v = coef[T.coef] * gg;
            break;
          }
          case J_DIFF_TENSOR:
            // (T G_a) . G_b
#pragma unroll
            for (int i = 0; i < DIM; ++i) {
              JT tg = JT(0);
#pragma unroll
              for (int j = 0; j < DIM; ++j) tg += coef[T.coef + i * DIM + j] * G[a][j];
              v += tg * G[b][i];
            }
            break;
          default:
            // phi_a-weighted vector . G_b
#pragma unroll
            for (int j = 0; j < DIM; ++j) v += coef[T.coef + a * DIM + j] * G[b][j];
            break;
        }
        if (T.slot != cur) {
          if (cur >= 0) {
            ej[(a * NL + b) * nslot + cur] = acc;
            if (P.all_mass && a != b) ej[(b * NL + a) * nslot + cur] = acc;
          }
          cur = T.slot;
          acc = JT(0);
        }
        acc += v;
      }
      if (cur >= 0) {
        ej[(a * NL + b) * nslot + cur] = acc;
        if (P.all_mass && a != b) ej[(b * NL + a) * nslot + cur] = acc;
      }
    }
  }
}

template <int DIM, int NS, class F>
__global__ void __launch_bounds__(128) k_volume(const VolumeParams P, const int begin, const int end,
                                                const int mode) {
  constexpr int NL = DIM + 1;
  constexpr int NQ = Rule<DIM>::NQ;
  const int k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;

  int nd[NL];
  F X[NL][DIM];
#pragma unroll
  for (int a = 0; a < NL; ++a) {
    const int v = P.verts[static_cast<int64_t>(k) * NL + a];
    nd[a] = P.nodes[static_cast<int64_t>(k) * NL + a];
#pragma unroll
    for (int d = 0; d < DIM; ++d) X[a][d] = P.coords[static_cast<int64_t>(v) * DIM + d];
  }
  // affine map x = X0 + Bm xi ; gradients of the P1 basis: rows of B^{-1} (local_operator.hh:461-464)
  F Bm[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) Bm[i][j] = X[j + 1][i] - X[0][i];
  F Bi[DIM][DIM];
  F det;
  // the inverse (basis gradients) only when a gradient, a flux or the Jacobian needs it: a
  // reaction-only residual pass needs |det| alone, and the FP64 division is the dearest
  // operation of the geometry (uniform branch)
  const bool need_inv = P.need_grad || P.has_flux || ((mode & 2) && P.J);
  if constexpr (DIM == 2) {
    det = Bm[0][0] * Bm[1][1] - Bm[0][1] * Bm[1][0];
    const F id = need_inv ? F(1) / det : F(0);
    if (need_inv) {
      Bi[0][0] = Bm[1][1] * id;  Bi[0][1] = -Bm[0][1] * id;
      Bi[1][0] = -Bm[1][0] * id; Bi[1][1] = Bm[0][0] * id;
    }
  } else {
    const F c00 = Bm[1][1] * Bm[2][2] - Bm[1][2] * Bm[2][1];
    const F c01 = Bm[1][2] * Bm[2][0] - Bm[1][0] * Bm[2][2];
    const F c02 = Bm[1][0] * Bm[2][1] - Bm[1][1] * Bm[2][0];
    det = Bm[0][0] * c00 + Bm[0][1] * c01 + Bm[0][2] * c02;
    const F id = need_inv ? F(1) / det : F(0);
    if (need_inv) {
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
  }
  const F adet = fabs(det);
  // the element volume only for programs that read entity_volume (an FP64 division)
  const F vol = P.need_vol ? adet / F(DIM == 2 ? 2 : 6) : F(0);
  F G[NL][DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    F s = 0.0;
#pragma unroll
    for (int kk = 0; kk < DIM; ++kk) {
      G[kk + 1][j] = need_inv ? Bi[kk][j] : F(0);
      s += G[kk + 1][j];
    }
    G[0][j] = -s;
  }

  const int bs = P.bs;
  F c[NL][NS];
#pragma unroll
  for (int a = 0; a < NL; ++a)
#pragma unroll
    for (int s = 0; s < NS; ++s) c[a][s] = P.x ? P.x[static_cast<int64_t>(nd[a]) * bs + s] : 0.0;
  // state gradients only when a program reads them or a term takes one (uniform branch)
  F g[NS][DIM];
#pragma unroll
  for (int s = 0; s < NS; ++s)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      F acc = 0.0;
      if (P.need_grad) {
#pragma unroll
        for (int a = 0; a < NL; ++a) acc += c[a][s] * G[a][j];
      }
      g[s][j] = acc;
    }

  const bool do_res = (mode & 1) && P.r;
  const bool do_jac = (mode & 2) && P.J;
  F rl[NL][NS];
#pragma unroll
  for (int a = 0; a < NL; ++a)
#pragma unroll
    for (int s = 0; s < NS; ++s) rl[a][s] = 0.0;
  // interpreter registers and Jacobian coefficients: per-thread slices of dynamic shared
  // memory (sized by the launcher from the program's registers and the term list)
  extern __shared__ __align__(16) unsigned char volume_smem[];
  F* const smem = reinterpret_cast<F*>(volume_smem);
  const Strided<F> R{smem + threadIdx.x, static_cast<int>(blockDim.x)};
  const Strided<F> coef{smem + static_cast<int64_t>(P.prog.nregs) * blockDim.x + threadIdx.x,
                        static_cast<int>(blockDim.x)};
  int ncoef = 0;
  if (do_jac) {
    for (int t = 0; t < P.n_jac_terms; ++t) {
      const Term T = P.jac_terms[t];
      // mass-type terms: nq point weights + the beta^2 S slot
      int sz = (T.kind == J_MASS || T.kind == J_MASS_U || T.kind == J_STORAGE_SELF) ? NQ + 1
             : (T.kind == J_DIFF_SCALAR) ? 1
             : (T.kind == J_DIFF_TENSOR) ? DIM * DIM
                                         : NL * DIM;
      ncoef = max(ncoef, T.coef + sz);
    }
    for (int i = 0; i < ncoef; ++i) coef[i] = 0.0;
  }
#pragma unroll 1
  for (int q = 0; q < NQ; ++q) {
    F u[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      F acc = 0.0;
#pragma unroll
      for (int a = 0; a < NL; ++a) acc += c[a][s] * phi_t<DIM, F>(q, a);
      u[s] = acc;
    }
    F xq[DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      F acc = X[0][i];
      if (P.need_pos) {
#pragma unroll
        for (int j = 0; j < DIM; ++j) acc += Bm[i][j] * xi_t<DIM, F>(q, j);
      }
      xq[i] = acc;
    }
    const F fq = static_cast<F>(Rule<DIM>::w(0)) * adet;
    for (int i = 0; i < P.prog.ninputs; ++i)
      R[i] = volume_input<DIM, NS, F>(P.prog.inputs[i], u, g, xq, F(P.t), vol, P.species_offset);
    run_program<F>(P.prog, P.tables, R);
    const uint8_t* out = P.prog.outputs;

    if (do_res) {
      F scal[NS], flux[NS][DIM];
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        scal[s] = 0.0;
#pragma unroll
        for (int j = 0; j < DIM; ++j) flux[s][j] = 0.0;
      }
      for (int t = 0; t < P.n_res_terms; ++t) {
        const Term T = P.res_terms[t];
        const F sc = F(T.form ? P.ca : P.cm);
        const F o = R[out[T.out]];
        F ds = 0.0, df[DIM];
#pragma unroll
        for (int j = 0; j < DIM; ++j) df[j] = 0.0;
        F ut = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
          if (s == T.test) ut = u[s];
        F gw[DIM];
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          gw[j] = 0.0;
#pragma unroll
          for (int s = 0; s < NS; ++s)
            if (s == T.trial) gw[j] = g[s][j];
        }
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
              F acc = 0.0;
#pragma unroll
              for (int j = 0; j < DIM; ++j) acc += R[out[T.out + i * DIM + j]] * gw[j];
              df[i] = -acc;
            }
            break;
          default: break;
        }
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          if (s == T.test) {
            scal[s] += sc * ds;
            if (P.has_flux) {
#pragma unroll
              for (int j = 0; j < DIM; ++j) flux[s][j] += sc * df[j];
            }
          }
        }
      }
      // rl[a][s] += (scal[s] phi_a - flux[s] . G_a) fq, with the factor fq applied once per
      // species rather than per entry (one FMA per entry for the scalar part)
      F ts[NS];
#pragma unroll
      for (int s = 0; s < NS; ++s) ts[s] = scal[s] * fq;
#pragma unroll
      for (int a = 0; a < NL; ++a) {
        const F pa = phi_t<DIM, F>(q, a);
#pragma unroll
        for (int s = 0; s < NS; ++s) rl[a][s] = fma(ts[s], pa, rl[a][s]);
      }
      if (P.has_flux) {
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          F tf[DIM];
#pragma unroll
          for (int j = 0; j < DIM; ++j) tf[j] = flux[s][j] * fq;
#pragma unroll
          for (int a = 0; a < NL; ++a) {
            F fg = 0.0;
#pragma unroll
            for (int j = 0; j < DIM; ++j) fg = fma(tf[j], G[a][j], fg);
            rl[a][s] -= fg;
          }
        }
      }
    }

    if (do_jac) {
      const F scm = F(P.cm) * fq, sca = F(P.ca) * fq;
      for (int t = 0; t < P.n_jac_terms; ++t) {
        const Term T = P.jac_terms[t];
        const F sc = T.form ? sca : scm;
        const F o = R[out[T.out]];
        F ut = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
          if (s == T.test) ut = u[s];
        switch (T.kind) {
          case J_MASS:
          case J_STORAGE_SELF: coef[T.coef + q] += sc * o; break;
          case J_MASS_U: coef[T.coef + q] += sc * o * ut; break;
          case J_DIFF_SCALAR: coef[T.coef] += sc * o; break;
          case J_DIFF_TENSOR:
#pragma unroll
            for (int i = 0; i < DIM * DIM; ++i) coef[T.coef + i] += sc * R[out[T.out + i]];
            break;
          case J_VELOCITY:
          case J_VELOCITY_JAC:
          case J_DIFFJAC_SCALAR:
          case J_DIFFJAC_TENSOR: {
            F vec[DIM];
            if (T.kind == J_VELOCITY) {
#pragma unroll
              for (int j = 0; j < DIM; ++j) vec[j] = -R[out[T.out + j]];
            } else if (T.kind == J_VELOCITY_JAC) {
#pragma unroll
              for (int j = 0; j < DIM; ++j) vec[j] = -R[out[T.out + j]] * ut;
            } else {
              F gw[DIM];
#pragma unroll
              for (int j = 0; j < DIM; ++j) {
                gw[j] = 0.0;
#pragma unroll
                for (int s = 0; s < NS; ++s)
                  if (s == T.trial) gw[j] = g[s][j];
              }
              if (T.kind == J_DIFFJAC_SCALAR) {
#pragma unroll
                for (int j = 0; j < DIM; ++j) vec[j] = o * gw[j];
              } else {
#pragma unroll
                for (int i = 0; i < DIM; ++i) {
                  F acc = 0.0;
#pragma unroll
                  for (int j = 0; j < DIM; ++j) acc += R[out[T.out + i * DIM + j]] * gw[j];
                  vec[i] = acc;
                }
              }
            }
#pragma unroll
            for (int a = 0; a < NL; ++a) {
              const F pa = phi_t<DIM, F>(q, a) * sc;
#pragma unroll
              for (int j = 0; j < DIM; ++j) coef[T.coef + a * DIM + j] += pa * vec[j];
            }
            break;
          }
          default: break;
        }
      }
    }
  }

  // element outputs: residual vector and Jacobian slot values, each written exactly once
  // (the gather kernels below add them into r and J in a fixed order)
  if (do_res) {
    double* er = P.er + static_cast<int64_t>(k) * NL * NS;
#pragma unroll
    for (int a = 0; a < NL; ++a)
#pragma unroll
      for (int s = 0; s < NS; ++s) er[a * NS + s] = static_cast<double>(rl[a][s]);
  }
  if (do_jac) {
    constexpr double be = MassConst<DIM>::beta;
    // mass-type terms: beta^2 S into the spare coefficient slot after the nq point weights
    for (int t = 0; t < P.n_jac_terms; ++t) {
      const Term T = P.jac_terms[t];
      if (T.kind == J_MASS || T.kind == J_MASS_U || T.kind == J_STORAGE_SELF) {
        F S = 0.0;
#pragma unroll
        for (int q = 0; q < NQ; ++q) S += coef[T.coef + q];
        coef[T.coef + NQ] = F(be * be) * S;
      }
    }
    const int64_t off = static_cast<int64_t>(k) * NL * NL * P.n_slots;
    if constexpr (std::is_same_v<F, float>) {
      // the FP32 Jacobian-only pass of the mixed-precision path
      element_jacobian<DIM, float>(P, coef, G, reinterpret_cast<float*>(P.ej) + off);
    } else if (P.jac_f32) {
      // mixed precision, computed alongside the fp64 residual: the element Jacobian in fp32
      // (the fp32 Krylov operator is built from it; the residual stays fp64)
      const StridedCast<F, float> cf{coef.p, coef.stride};
      float Gf[NL][DIM];
#pragma unroll
      for (int a = 0; a < NL; ++a)
#pragma unroll
        for (int j = 0; j < DIM; ++j) Gf[a][j] = static_cast<float>(G[a][j]);
      element_jacobian<DIM, float>(P, cf, Gf, reinterpret_cast<float*>(P.ej) + off);
    } else {
      element_jacobian<DIM, double>(P, coef, G, P.ej + off);
    }
  }
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
  if (o.sell) o.sell[o.sell_bpos[blk] * bs2 + slot_pos[m]] = static_cast<float>(v);
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
