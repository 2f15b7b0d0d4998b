// Volume element kernel: residual and analytic Jacobian of the mass and stiffness forms of
// one cell (dune/copasi/model/diffusion_reaction/local_operator.hh:417-491, 541-707).
//
// The body is a template over a Spec that supplies the cell's term lists and evaluates
// the model's expression program at a quadrature point.  Two Specs exist:
//   * the library's interpreter Spec (assemble_volume.cu): terms read from device memory,
//     the bytecode run by the device interpreter with its register file in shared memory;
//   * a Spec generated at model set-up (volume_jit.cpp): terms as compile-time tables and
//     the program as straight-line code, compiled with NVRTC for sm_103a, so the term
//     loops unroll and the registers and coefficients live in registers.
// This header is compiled by nvcc and by NVRTC: it includes nothing but device.cuh (whose
// only standard header, <cstdint>, NVRTC receives as a stub).
#pragma once

#include "device.cuh"

namespace dcgpu {
namespace vk {

template <class A, class B>
struct same_type {
  static constexpr bool value = false;
};
template <class A>
struct same_type<A, A> {
  static constexpr bool value = true;
};

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

// Both rules have one point per vertex: point q carries the large barycentric weight
// alpha at vertex vertex_of<DIM>(q) and beta elsewhere, so phi_a(q) phi_b(q) =
// beta^2 + beta (alpha - beta) ([a = v(q)] + [b = v(q)]) + (alpha - beta)^2 [a = b = v(q)].
// A mass-type element matrix sum_q c_q phi_a(q) phi_b(q) is then
// beta^2 S + k1 (c_a + c_b) + [a = b] k2 c_a with S = sum_q c_q and c_a the weight of the
// point at vertex a: two additions per entry instead of NQ multiply-adds.
template <int DIM> struct MassConst;
template <> struct MassConst<2> {
  static constexpr double alpha = 2.0 / 3.0, beta = 1.0 / 6.0;
};
template <> struct MassConst<3> {
  static constexpr double alpha = 0.5854101966249685, beta = 0.1381966011250105;
};

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
__host__ __device__ constexpr PhiTable<DIM, F> make_phi_table() {
  PhiTable<DIM, F> t{};
  for (int q = 0; q < Rule<DIM>::NQ; ++q)
    for (int a = 0; a <= DIM; ++a) t.v[q][a] = static_cast<F>(phi_value<DIM>(q, a));
  return t;
}
static __constant__ PhiTable<2, double> c_phi2d = make_phi_table<2, double>();
static __constant__ PhiTable<3, double> c_phi3d = make_phi_table<3, double>();
static __constant__ PhiTable<2, float> c_phi2f = make_phi_table<2, float>();
static __constant__ PhiTable<3, float> c_phi3f = make_phi_table<3, float>();

template <int DIM, class F>
__device__ __forceinline__ F phi_t(int q, int a) {
  if constexpr (same_type<F, double>::value) return DIM == 2 ? c_phi2d.v[q][a] : c_phi3d.v[q][a];
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
template <int DIM>
__device__ __forceinline__ constexpr int point_of_vertex(int a) {
  // 2D: points 0, 1, 2 sit at vertices 1, 2, 0; 3D: point q at vertex q
  return DIM == 2 ? (a == 0 ? 2 : a - 1) : a;
}
template <int DIM>
__device__ __forceinline__ constexpr int vertex_of_point(int q) {
  return DIM == 2 ? (q == 2 ? 0 : q + 1) : q;
}

// value of program input `id` at a point (species values / gradients relative to the
// compartment's first species, positions, time, entity volume)
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
template <int DIM, class JT, class Spec, class Coef, class Sink>
__device__ __forceinline__ void element_jacobian_to(const VolumeParams& P, Coef coef, const JT (&G)[DIM + 1][DIM],
                                                    Sink sink) {
  constexpr int NL = DIM + 1;
  constexpr int NQ = Rule<DIM>::NQ;
  constexpr double al = MassConst<DIM>::alpha, be = MassConst<DIM>::beta;
  const JT k1 = static_cast<JT>(be * (al - be)), k2 = static_cast<JT>((al - be) * (al - be));
  const int nslot = Spec::n_slots(P);
  const bool all_mass = Spec::all_mass(P);
#pragma unroll
  for (int a = 0; a < NL; ++a) {
#pragma unroll
    for (int b = 0; b < NL; ++b) {
      if (all_mass && b < a) continue;
      int cur = -1;
      JT acc = JT(0);
#pragma unroll
      for (int t = 0; t < Spec::n_jac(P); ++t) {
        const Term T = Spec::jac(P, t);
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
          if (cur >= 0) sink(a, b, cur, acc, all_mass && a != b);
          cur = T.slot;
          acc = JT(0);
        }
        acc += v;
      }
      if (cur >= 0) sink(a, b, cur, acc, all_mass && a != b);
    }
  }
  (void)nslot;
}

// the element matrix stored per slot: ej[(a * NL + b) * n_slots + slot] (and the mirrored
// pair of a symmetric all-mass matrix)
template <int DIM, class JT, class Spec, class Coef>
__device__ __forceinline__ void element_jacobian(const VolumeParams& P, Coef coef, const JT (&G)[DIM + 1][DIM],
                                                 JT* ej) {
  constexpr int NL = DIM + 1;
  const int nslot = Spec::n_slots(P);
  element_jacobian_to<DIM, JT, Spec>(P, coef, G, [&](int a, int b, int slot, JT acc, bool mirror) {
    ej[(a * NL + b) * nslot + slot] = acc;
    if (mirror) ej[(b * NL + a) * nslot + slot] = acc;
  });
}

// the element matrix applied to the direction v at the element's block rows nd:
// out[a][test] += J_e(a test, b trial) v(nd[b] trial) (matrix-free Jacobian products)
template <int DIM, int NS, class JT, class Spec, class Coef>
__device__ __forceinline__ void element_jacobian_apply(const VolumeParams& P, Coef coef, const JT (&G)[DIM + 1][DIM],
                                                       const int (&nd)[DIM + 1], JT (&out)[DIM + 1][NS]) {
  const int bs = P.bs;
  element_jacobian_to<DIM, JT, Spec>(P, coef, G, [&](int a, int b, int slot, JT acc, bool mirror) {
    const int pos = P.slot_pos[slot];
    const int te = pos / bs, tr = pos - te * bs;
    const JT vb = static_cast<JT>(P.v[static_cast<int64_t>(nd[b]) * bs + tr]);
    const JT va = mirror ? static_cast<JT>(P.v[static_cast<int64_t>(nd[a]) * bs + tr]) : JT(0);
#pragma unroll
    for (int s = 0; s < NS; ++s)
      if (s == te) {
        out[a][s] += acc * vb;
        if (mirror) out[b][s] += acc * va;
      }
  });
}

// The element kernel body for cell k.  R: the program's register file, coef: the
// element's Jacobian coefficients (shared-memory slices for the interpreter, local arrays
// indexed by constants for generated Specs).  MODE: 1 residual, 2 Jacobian, 3 both, or 0
// for the run-time `mode` argument.  er_dst / ej_dst: where the cell's residual vector and
// Jacobian slot values go (a staging record in shared memory), or null for their places in
// P.er / P.ej.  verts_src / nodes_src: the cell's vertex and block-row indices already staged
// in shared memory, or null to read them from P.verts / P.nodes.
template <int DIM, int NS, class F, class Spec, int MODE, class Regs, class Coef>
__device__ __forceinline__ void volume_element(const VolumeParams& P, const int k, const int mode_rt, Regs R,
                                               Coef coef, double* er_dst = nullptr, void* ej_dst = nullptr,
                                               const int32_t* verts_src = nullptr,
                                               const int32_t* nodes_src = nullptr) {
  constexpr int NL = DIM + 1;
  constexpr int NQ = Rule<DIM>::NQ;
  const int mode = MODE ? MODE : mode_rt;

  int nd[NL];
  F X[NL][DIM];
#pragma unroll
  for (int a = 0; a < NL; ++a) {
    const int v = verts_src ? verts_src[a] : P.verts[static_cast<int64_t>(k) * NL + a];
    nd[a] = nodes_src ? nodes_src[a] : P.nodes[static_cast<int64_t>(k) * NL + a];
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
  const bool do_apply = (mode & 8) != 0;  // matrix-free J v (kVolumeJacobianApply)
  const bool need_inv = Spec::need_grad(P) || Spec::has_flux(P) || ((mode & 2) && P.J) || do_apply;
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
  const F vol = Spec::need_vol(P) ? adet / F(DIM == 2 ? 2 : 6) : F(0);
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
      if (Spec::need_grad(P)) {
#pragma unroll
        for (int a = 0; a < NL; ++a) acc += c[a][s] * G[a][j];
      }
      g[s][j] = acc;
    }

  const bool do_res = (mode & 1) && P.r;
  const bool do_jac = ((mode & 2) && P.J) || do_apply;
  const bool jac_prog = (mode & 2) != 0;  // which program and residual term list the pass runs
  // Every point of the rule sits at one vertex: phi_a(q) = beta + (alpha - beta) [a = v(q)].
  // So the value of species s at point q is beta sum_a c_a + (alpha - beta) c_v(q), and the
  // scalar residual part sum_q w_q phi_a(q) = beta sum_q w_q + (alpha - beta) w_q(a): one
  // FMA per value instead of NL, and the point sums folded once per cell.
  constexpr F kBe = static_cast<F>(MassConst<DIM>::beta);
  constexpr F kAmB = static_cast<F>(MassConst<DIM>::alpha - MassConst<DIM>::beta);
  F bsum[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    F acc = c[0][s];
#pragma unroll
    for (int a = 1; a < NL; ++a) acc += c[a][s];
    bsum[s] = kBe * acc;
  }
  // residual accumulators: the scalar part of the point at each vertex, its sum over the
  // points, and the flux summed over the points (the basis gradients are constant on a cell)
  F rl[NL][NS], tsum[NS], fsum[NS][DIM];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    tsum[s] = 0.0;
#pragma unroll
    for (int a = 0; a < NL; ++a) rl[a][s] = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j) fsum[s][j] = 0.0;
  }
  int ncoef = 0;
  if (do_jac) {
#pragma unroll
    for (int t = 0; t < Spec::n_jac(P); ++t) {
      const Term T = Spec::jac(P, t);
      // mass-type terms: nq point weights + the beta^2 S slot
      int sz = (T.kind == J_MASS || T.kind == J_MASS_U || T.kind == J_STORAGE_SELF) ? NQ + 1
             : (T.kind == J_DIFF_SCALAR) ? 1
             : (T.kind == J_DIFF_TENSOR) ? DIM * DIM
                                         : NL * DIM;
      ncoef = max(ncoef, T.coef + sz);
    }
#pragma unroll
    for (int i = 0; i < Spec::coef_bound(P, ncoef); ++i) coef[i] = 0.0;
  }
  auto point = [&](const int q) {
    const int vq = vertex_of_point<DIM>(q);
    F u[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      F cv = c[0][s];
#pragma unroll
      for (int a = 1; a < NL; ++a)
        if (a == vq) cv = c[a][s];
      u[s] = fma(kAmB, cv, bsum[s]);
    }
    F xq[DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      F acc = X[0][i];
      if (Spec::need_pos(P)) {
#pragma unroll
        for (int j = 0; j < DIM; ++j) acc += Bm[i][j] * xi_t<DIM, F>(q, j);
      }
      xq[i] = acc;
    }
    const F fq = static_cast<F>(Rule<DIM>::w(0)) * adet;
    Spec::template run<DIM, NS, F>(P, jac_prog, R, u, g, xq, F(P.t), vol);

    if (do_res) {
      F scal[NS], flux[NS][DIM];
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        scal[s] = 0.0;
#pragma unroll
        for (int j = 0; j < DIM; ++j) flux[s][j] = 0.0;
      }
#pragma unroll
      for (int t = 0; t < Spec::n_res(P, jac_prog); ++t) {
        const Term T = Spec::res(P, jac_prog, t);
        const F sc = F(T.form ? P.ca : P.cm);
        const F o = R[Spec::out(P, jac_prog, T.out)];
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
            for (int j = 0; j < DIM; ++j) df[j] = R[Spec::out(P, jac_prog, T.out + j)] * ut;
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
              for (int j = 0; j < DIM; ++j) acc += R[Spec::out(P, jac_prog, T.out + i * DIM + j)] * gw[j];
              df[i] = -acc;
            }
            break;
          default: break;
        }
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          if (s == T.test) {
            scal[s] += sc * ds;
            if (Spec::has_flux(P)) {
#pragma unroll
              for (int j = 0; j < DIM; ++j) flux[s][j] += sc * df[j];
            }
          }
        }
      }
      // per point only sums: the point's scalar part goes to its vertex, its total and the
      // flux total accumulate (the weights and gradients are applied after the last point)
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        tsum[s] += scal[s];
#pragma unroll
        for (int a = 0; a < NL; ++a)
          if (a == vq) rl[a][s] = scal[s];
      }
      if (Spec::has_flux(P)) {
#pragma unroll
        for (int s = 0; s < NS; ++s)
#pragma unroll
          for (int j = 0; j < DIM; ++j) fsum[s][j] += flux[s][j];
      }
    }

    if (do_jac) {
      const F scm = F(P.cm) * fq, sca = F(P.ca) * fq;
#pragma unroll
      for (int t = 0; t < Spec::n_jac(P); ++t) {
        const Term T = Spec::jac(P, t);
        const F sc = T.form ? sca : scm;
        const F o = R[Spec::out(P, true, T.out)];
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
            for (int i = 0; i < DIM * DIM; ++i) coef[T.coef + i] += sc * R[Spec::out(P, true, T.out + i)];
            break;
          case J_VELOCITY:
          case J_VELOCITY_JAC:
          case J_DIFFJAC_SCALAR:
          case J_DIFFJAC_TENSOR: {
            F vec[DIM];
            if (T.kind == J_VELOCITY) {
#pragma unroll
              for (int j = 0; j < DIM; ++j) vec[j] = -R[Spec::out(P, true, T.out + j)];
            } else if (T.kind == J_VELOCITY_JAC) {
#pragma unroll
              for (int j = 0; j < DIM; ++j) vec[j] = -R[Spec::out(P, true, T.out + j)] * ut;
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
                  for (int j = 0; j < DIM; ++j) acc += R[Spec::out(P, true, T.out + i * DIM + j)] * gw[j];
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
  };
  // the interpreter keeps the point loop rolled (its body is large); generated Specs unroll
  // it, so every coefficient index is a constant and the coefficients stay in registers
  if constexpr (Spec::kUnrollPoints) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) point(q);
  } else {
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) point(q);
  }

  // rl[a][s] = fq (sum_q scal_q phi_a(q) - fsum . G_a), all points having the weight fq
  if (do_res) {
    const F fq = static_cast<F>(Rule<DIM>::w(0)) * adet;
    const F fb = fq * kBe, fab = fq * kAmB;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const F base = fb * tsum[s];
#pragma unroll
      for (int a = 0; a < NL; ++a) rl[a][s] = fma(fab, rl[a][s], base);
      if (Spec::has_flux(P)) {
        F tf[DIM];
#pragma unroll
        for (int j = 0; j < DIM; ++j) tf[j] = fsum[s][j] * fq;
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

  // element outputs: residual vector and Jacobian slot values, each written exactly once
  // (the gather kernels add them into r and J in a fixed order)
  if (do_res) {
    double* er = er_dst ? er_dst : P.er + static_cast<int64_t>(k) * NL * NS;
#pragma unroll
    for (int a = 0; a < NL; ++a)
#pragma unroll
      for (int s = 0; s < NS; ++s) er[a * NS + s] = static_cast<double>(rl[a][s]);
  }
  if (do_jac) {
    constexpr double be = MassConst<DIM>::beta;
    // mass-type terms: beta^2 S into the spare coefficient slot after the nq point weights
#pragma unroll
    for (int t = 0; t < Spec::n_jac(P); ++t) {
      const Term T = Spec::jac(P, t);
      if (T.kind == J_MASS || T.kind == J_MASS_U || T.kind == J_STORAGE_SELF) {
        F S = 0.0;
#pragma unroll
        for (int q = 0; q < NQ; ++q) S += coef[T.coef + q];
        coef[T.coef + NQ] = F(be * be) * S;
      }
    }
    const int64_t off = ej_dst ? 0 : static_cast<int64_t>(k) * NL * NL * Spec::n_slots(P);
    void* const ejb = ej_dst ? ej_dst : static_cast<void*>(P.ej);
    if (do_apply) {
      F out[NL][NS];
#pragma unroll
      for (int a = 0; a < NL; ++a)
#pragma unroll
        for (int s = 0; s < NS; ++s) out[a][s] = F(0);
      element_jacobian_apply<DIM, NS, F, Spec>(P, coef, G, nd, out);
      double* er = er_dst ? er_dst : P.er + static_cast<int64_t>(k) * NL * NS;
#pragma unroll
      for (int a = 0; a < NL; ++a)
#pragma unroll
        for (int s = 0; s < NS; ++s) er[a * NS + s] = static_cast<double>(out[a][s]);
    } else if constexpr (same_type<F, float>::value) {
      // the FP32 Jacobian-only pass of the mixed-precision path
      element_jacobian<DIM, float, Spec>(P, coef, G, static_cast<float*>(ejb) + off);
    } else if (P.jac_f32) {
      // mixed precision, computed alongside the fp64 residual: the element Jacobian in fp32
      // (the fp32 Krylov operator is built from it; the residual stays fp64)
      const auto cf = Spec::template as_float<F>(coef);
      float Gf[NL][DIM];
#pragma unroll
      for (int a = 0; a < NL; ++a)
#pragma unroll
        for (int j = 0; j < DIM; ++j) Gf[a][j] = static_cast<float>(G[a][j]);
      element_jacobian<DIM, float, Spec>(P, cf, Gf, static_cast<float*>(ejb) + off);
    } else {
      element_jacobian<DIM, double, Spec>(P, coef, G, static_cast<double*>(ejb) + off);
    }
  }
}

}  // namespace vk
}  // namespace dcgpu

namespace dcgpu {
namespace vk {

// A thread's local arrays for generated Specs: every index is a constant once the term and
// point loops are unrolled, so the arrays live in registers
template <class F>
struct Arr {
  F* p;
  __device__ __forceinline__ F& operator[](int i) const { return p[i]; }
};
template <class F>
struct ArrCast {
  const F* p;
  __device__ __forceinline__ float operator[](int i) const { return static_cast<float>(p[i]); }
};

// copy n elements of T from a shared-memory staging area of per-thread records (record
// length REC, stride REC + 1) to consecutive global memory: each global store of a warp
// covers consecutive addresses
template <class T, int REC>
__device__ __forceinline__ void stage_out(const T* __restrict__ stage, T* __restrict__ dst, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i / REC, e = i - t * REC;
    dst[i] = stage[t * (REC + 1) + e];
  }
}

constexpr int kJitThreads = 128;

// ---- bulk asynchronous copies (the TMA engine) of the block's element index data
// One thread of the block arms an mbarrier with the expected byte count and issues
// cp.async.bulk copies global -> shared; every thread then waits on the barrier's phase.
// The wait is bounded: after kBulkWaitPolls unsuccessful polls the block reports failure and
// its threads read the indices from global memory instead (the result is the same).
constexpr int kBulkWaitPolls = 1 << 20;

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
// bytes (a multiple of 16) from 16-byte aligned global src to 16-byte aligned shared dst
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// true once phase `parity` of the barrier has completed, false after kBulkWaitPolls polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  for (int i = 0; i < kBulkWaitPolls; ++i) {
    unsigned done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// largest staging area the compiled volume kernels use (larger records are not staged)
constexpr int kJitStageMax = 160 * 1024;

// bytes of dynamic shared memory of a k_volume_jit launch: the staged residual records
// (NL * NS doubles per thread) and Jacobian records (NL * NL * nslot values of esize bytes)
__host__ __device__ constexpr int jit_stage_bytes(int dim, int ns, int nslot, int mode, int esize) {
  return ((mode & 1) ? kJitThreads * ((dim + 1) * ns + 1) * 8 : 0) +
         ((mode & 2) ? kJitThreads * ((dim + 1) * (dim + 1) * nslot + 1) * esize : 0);
}

// Kernel of a generated Spec S (instantiated only by the run-time compiled sources): one
// thread per cell, MODE fixed at compile time.  The cells' element outputs are staged in
// shared memory and written out as one contiguous range per block: a thread's own record
// is contiguous but records are strided across the warp, so direct stores would each touch
// 32 sectors and throttle the store pipe.
template <int DIM, int NS, class F, class S, int MODE>
__global__ void __launch_bounds__(kJitThreads) k_volume_jit(const VolumeParams P, const int begin, const int end) {
  constexpr int NL = DIM + 1;
  constexpr int RE = NL * NS;
  constexpr int RJ = NL * NL * S::kSlots;
  const int k0 = begin + blockIdx.x * kJitThreads;
  const int k = k0 + threadIdx.x;
  if constexpr (!S::kStage) {
    // records too large to stage: each thread writes its own
    if (k < end) {
      F R[S::kRegs];
      F C[S::kCoefs];
      volume_element<DIM, NS, F, S, MODE>(P, k, MODE, Arr<F>{R}, Arr<F>{C});
    }
  } else {
    extern __shared__ __align__(16) unsigned char jit_stage[];
    double* const ser = reinterpret_cast<double*>(jit_stage);
    unsigned char* const sej = jit_stage + ((MODE & 1) ? kJitThreads * (RE + 1) * 8 : 0);
    const bool ej32 = same_type<F, float>::value || P.jac_f32;
    // the block's cells are consecutive: their vertex and block-row indices are two
    // contiguous ranges, brought into shared memory by the bulk-copy engine
    __shared__ __align__(16) int32_t s_verts[kJitThreads * NL];
    __shared__ __align__(16) int32_t s_nodes[kJitThreads * NL];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_bulk;
    const int nv = min(kJitThreads, end - k0);
    const int32_t* gv = P.verts + static_cast<int64_t>(k0) * NL;
    const int32_t* gn = P.nodes + static_cast<int64_t>(k0) * NL;
    const unsigned bytes = static_cast<unsigned>(nv * NL * 4);
    const bool bulk = bytes % 16 == 0 && (reinterpret_cast<uintptr_t>(gv) & 15) == 0 &&
                      (reinterpret_cast<uintptr_t>(gn) & 15) == 0;
    if (threadIdx.x == 0) {
      s_bulk = 0;
      if (bulk) {
        mbar_init(&s_bar, 1);
        mbar_expect_tx(&s_bar, 2 * bytes);
        bulk_load(s_verts, gv, bytes, &s_bar);
        bulk_load(s_nodes, gn, bytes, &s_bar);
      }
    }
    __syncthreads();
    bool staged = false;
    if (bulk) {
      staged = mbar_wait(&s_bar, 0);
      if (!staged) atomicExch(&s_bulk, 1);
    }
    __syncthreads();
    // a wait that gave up in any thread: every thread reads its indices from global memory
    // (the copies still land in the block's own shared memory before it exits below)
    if (s_bulk) staged = false;
    if (k < end) {
      F R[S::kRegs];
      F C[S::kCoefs];
      volume_element<DIM, NS, F, S, MODE>(
          P, k, MODE, Arr<F>{R}, Arr<F>{C}, (MODE & 1) ? ser + threadIdx.x * (RE + 1) : nullptr,
          (MODE & 2) ? static_cast<void*>(sej + threadIdx.x * (RJ + 1) * (ej32 ? 4 : 8)) : nullptr,
          staged ? s_verts + threadIdx.x * NL : nullptr, staged ? s_nodes + threadIdx.x * NL : nullptr);
    }
    if (bulk && s_bulk && threadIdx.x == 0) mbar_wait(&s_bar, 0);  // the copies in flight, bounded
    __syncthreads();
    if ((MODE & 1) && P.r) stage_out<double, RE>(ser, P.er + static_cast<int64_t>(k0) * RE, nv * RE);
    if ((MODE & 2) && P.J) {
      if (ej32)
        stage_out<float, RJ>(reinterpret_cast<const float*>(sej),
                             reinterpret_cast<float*>(P.ej) + static_cast<int64_t>(k0) * RJ, nv * RJ);
      else
        stage_out<double, RJ>(reinterpret_cast<const double*>(sej), P.ej + static_cast<int64_t>(k0) * RJ, nv * RJ);
    }
  }
}

}  // namespace vk
}  // namespace dcgpu
