#include "mcolor.hpp"

#include <stdexcept>
#include <string>
#include <type_traits>

#include "blockops.cuh"
#include "graph.hpp"
#include "linalg.cuh"
#include "sellrow.cuh"

namespace dcgpu {

namespace {

constexpr int kT = 128;

inline int grid_for(int64_t n) {
  int64_t b = (n + kT - 1) / kT;
  return static_cast<int>(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

__device__ __forceinline__ bool skip(const double* sc, int slot) { return sc && sc[slot] != 0.0; }

__global__ void k_inverse_positions(int64_t n, const int32_t* __restrict__ perm, int32_t* __restrict__ ipos) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += stride)
    ipos[perm[p]] = static_cast<int32_t>(p);
}

// One colour of a sweep, a thread per block row i of colour c:
//   t = base - sum over j in S of A_ij z_j
// kSorFirst   base r_i,        S lower,     z_i  = omega Dinv_i t   (first forward SOR sweep, z = 0)
// kSorFull    base r_i,        S all,       z_i += omega Dinv_i t   (SOR sweep)
// kLowerSolve base omega r_i,  S lower,     z_i  = t                (ILU forward, unit L)
// kUpperSolve base z_i,        S upper,     z_i  = Uinv_i t         (ILU backward)
// kDiluLower  base omega r_i,  S lower,     z_i  = Dinv_i t
// kDiluUpper  base 0,          S upper,     z_i += Dinv_i t
// "lower" / "upper": columns of an earlier / later colour (a proper colouring puts no other
// row of colour c in row i).  dmat holds the inverse pivot blocks of the mode.
enum SweepMode : int { kSorFirst = 0, kSorFull = 1, kLowerSolve = 2, kUpperSolve = 3, kDiluLower = 4, kDiluUpper = 5 };

template <int B, class T, int MODE>
__global__ void __launch_bounds__(kT) k_sweep(Sell S, const int32_t* __restrict__ colour, int c,
                                              const T* __restrict__ vals, const T* __restrict__ dmat,
                                              const T* __restrict__ r, T* __restrict__ z, T omega, const double* sc,
                                              int slot) {
  if (skip(sc, slot)) return;
  const SliceLoop L;
  for (int64_t sl = L.first; sl < S.nslices; sl += L.stride) {
    const int64_t i = sl * 32 + L.lane;
    if (i >= S.nrows || colour[i] != c) continue;
    const int64_t oi = i * B;
    T t[B];
#pragma unroll
    for (int s = 0; s < B; ++s) {
      if (MODE == kSorFirst || MODE == kSorFull) t[s] = r[oi + s];
      else if (MODE == kLowerSolve || MODE == kDiluLower) t[s] = omega * r[oi + s];
      else if (MODE == kUpperSolve) t[s] = z[oi + s];
      else t[s] = T(0);
    }
    T acc[B];
#pragma unroll
    for (int s = 0; s < B; ++s) acc[s] = T(0);
    sell_row_apply<B, T>(
        S, sl, L.lane, vals,
        [&](int32_t j) {
          if (MODE == kSorFull) return true;
          const int cj = colour[j];
          return (MODE == kSorFirst || MODE == kLowerSolve || MODE == kDiluLower) ? cj < c : cj > c;
        },
        [&](int32_t j, T (&xv)[B]) {
#pragma unroll
          for (int q = 0; q < B; ++q) xv[q] = z[static_cast<int64_t>(j) * B + q];
        },
        acc);
#pragma unroll
    for (int s = 0; s < B; ++s) t[s] -= acc[s];
    if (MODE == kLowerSolve) {
#pragma unroll
      for (int s = 0; s < B; ++s) z[oi + s] = t[s];
      continue;
    }
    const T* d = dmat + i * B * B;
    T out[B];
#pragma unroll
    for (int s = 0; s < B; ++s) {
      T a = T(0);
#pragma unroll
      for (int q = 0; q < B; ++q) a += d[s * B + q] * t[q];
      out[s] = a;
    }
#pragma unroll
    for (int s = 0; s < B; ++s) {
      if (MODE == kSorFirst) z[oi + s] = omega * out[s];
      else if (MODE == kSorFull) z[oi + s] = z[oi + s] + omega * out[s];
      else if (MODE == kDiluUpper) z[oi + s] = z[oi + s] + out[s];
      else z[oi + s] = out[s];
    }
  }
}

// ILU(0) rows of one colour (IKJ order on the colour-ordered matrix): for every earlier row k
// of row i's pattern, in increasing colour order position, L_ik = A_ik Uinv_k and A_ij -= L_ik
// U_kj for the later columns j of row k that row i's pattern holds; then Uinv_i = A_ii^-1.
// Rows k belong to earlier colours, whose factors are final.
template <int B>
__global__ void __launch_bounds__(kT) k_ilu0(int64_t begin, int64_t end, const int32_t* __restrict__ perm,
                                             const int32_t* __restrict__ ipos, const int32_t* __restrict__ rowptr,
                                             const int32_t* __restrict__ colidx, const int32_t* __restrict__ diag,
                                             double* __restrict__ lu, double* __restrict__ uinv, int* status) {
  constexpr int BB = B * B;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t p = begin + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < end; p += stride) {
    const int32_t i = perm[p];
    const int32_t b0 = rowptr[i], b1 = rowptr[i + 1];
    int32_t last = -1;
    for (;;) {
      int32_t eb = -1, qb = 0x7fffffff;
      for (int32_t e = b0; e < b1; ++e) {
        const int32_t q = ipos[colidx[e]];
        if (q < p && q > last && q < qb) {
          qb = q;
          eb = e;
        }
      }
      if (eb < 0) break;
      last = qb;
      const int32_t k = colidx[eb];
      double a[B][B], u[B][B], l[B][B];
      load_block<B>(lu + static_cast<int64_t>(eb) * BB, a);
      load_block<B>(uinv + static_cast<int64_t>(k) * BB, u);
      mul_block<B>(a, u, l);
      store_block<B>(lu + static_cast<int64_t>(eb) * BB, l);
      for (int32_t f = rowptr[k]; f < rowptr[k + 1]; ++f) {
        const int32_t j = colidx[f];
        if (ipos[j] <= qb) continue;
        for (int32_t g = b0; g < b1; ++g) {
          if (colidx[g] != j) continue;
          double c[B][B];
          load_block<B>(lu + static_cast<int64_t>(g) * BB, c);
          sub_mul_block<B>(l, lu + static_cast<int64_t>(f) * BB, c);
          store_block<B>(lu + static_cast<int64_t>(g) * BB, c);
          break;
        }
      }
    }
    double a[B][B], inv[B][B];
    load_block<B>(lu + static_cast<int64_t>(diag[i]) * BB, a);
    if (!invert_block<B>(a, inv)) {
      atomicExch(status, 1);
      continue;
    }
    store_block<B>(uinv + static_cast<int64_t>(i) * BB, inv);
  }
}

// DILU pivots of one colour: D_i = A_ii - sum over earlier rows k of A_ik D_k^-1 A_ki
template <int B>
__global__ void __launch_bounds__(kT) k_dilu(int64_t begin, int64_t end, const int32_t* __restrict__ perm,
                                             const int32_t* __restrict__ ipos, const int32_t* __restrict__ rowptr,
                                             const int32_t* __restrict__ colidx, const int32_t* __restrict__ diag,
                                             const double* __restrict__ vals, double* __restrict__ dinv, int* status) {
  constexpr int BB = B * B;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t p = begin + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < end; p += stride) {
    const int32_t i = perm[p];
    double d[B][B];
    load_block<B>(vals + static_cast<int64_t>(diag[i]) * BB, d);
    for (int32_t e = rowptr[i]; e < rowptr[i + 1]; ++e) {
      const int32_t k = colidx[e];
      if (ipos[k] >= p) continue;
      for (int32_t f = rowptr[k]; f < rowptr[k + 1]; ++f) {
        if (colidx[f] != i) continue;
        double a[B][B], dk[B][B], t[B][B];
        load_block<B>(vals + static_cast<int64_t>(e) * BB, a);
        load_block<B>(dinv + static_cast<int64_t>(k) * BB, dk);
        mul_block<B>(a, dk, t);
        sub_mul_block<B>(t, vals + static_cast<int64_t>(f) * BB, d);
        break;
      }
    }
    double inv[B][B];
    if (!invert_block<B>(d, inv)) {
      atomicExch(status, 1);
      continue;
    }
    store_block<B>(dinv + static_cast<int64_t>(i) * BB, inv);
  }
}

template <class T>
__global__ void k_scale(int64_t n, const T* __restrict__ r, T* __restrict__ z, double omega, const double* sc,
                        int slot) {
  if (skip(sc, slot)) return;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    z[i] = static_cast<T>(omega * static_cast<double>(r[i]));
}

}  // namespace

void ColorPrecond::build(Kind kind, int64_t nrows, int bs, int64_t nnzb, const int32_t* rowptr,
                         const int32_t* colidx, const int32_t* diag, cudaStream_t s) {
  if (bs < 1 || bs > 8) throw std::runtime_error("multicolour preconditioner: block size " + std::to_string(bs) +
                                                 " unsupported");
  kind_ = kind;
  n_ = nrows;
  nnzb_ = nnzb;
  bs_ = bs;
  rowptr_ = rowptr;
  colidx_ = colidx;
  diag_ = diag;
  colour_.resize(static_cast<size_t>(nrows));
  perm_.resize(static_cast<size_t>(nrows));
  ipos_.resize(static_cast<size_t>(nrows));
  DeviceGraph g;
  g.n = nrows;
  g.rowptr = rowptr;
  g.colidx = colidx;
  const int nc = color_rows(g, colour_.get(), s);
  order_by_color(nrows, colour_.get(), nc, perm_.get(), &offsets_, s);
  count_launches(1);
  k_inverse_positions<<<grid_for(nrows), kT, 0, s>>>(nrows, perm_.get(), ipos_.get());
  sell_structure(nrows, rowptr, colidx, &sell_, s);
  const size_t nb2 = static_cast<size_t>(bs) * bs;
  if (kind == Kind::Ilu0) {
    lu_.resize(static_cast<size_t>(nnzb) * nb2);
    dfac_.resize(static_cast<size_t>(nrows) * nb2);
  } else if (kind == Kind::Dilu) {
    dfac_.resize(static_cast<size_t>(nrows) * nb2);
  }
  cuda_check(cudaStreamSynchronize(s), "multicolour set-up");
}

void ColorPrecond::setup(const double* vals, const double* dinv, const float* dinv32, bool fp32, int* status,
                         cudaStream_t s, const Sell* sell_ext, const float* sv32_ext) {
  dinv_ = dinv;
  dinv32_ = dinv32;
  fp32_ = fp32;
  const int nc = colors();
  const size_t nb2 = static_cast<size_t>(bs_) * bs_;
  if (kind_ == Kind::Ilu0) {
    cuda_check(cudaMemcpyAsync(lu_.get(), vals, nnzb_ * nb2 * sizeof(double), cudaMemcpyDeviceToDevice, s), "ilu");
    for (int c = 0; c < nc; ++c) {
      const int64_t b = offsets_[c], e = offsets_[c + 1];
      if (e == b) continue;
      count_launches(1);
#define DC_ILU(B)                                                                                                 \
  case B:                                                                                                         \
    k_ilu0<B><<<grid_for(e - b), kT, 0, s>>>(b, e, perm_.get(), ipos_.get(), rowptr_, colidx_, diag_, lu_.get(), \
                                             dfac_.get(), status);                                                \
    break;
      switch (bs_) { DC_ILU(1) DC_ILU(2) DC_ILU(3) DC_ILU(4) DC_ILU(5) DC_ILU(6) DC_ILU(7) DC_ILU(8) }
#undef DC_ILU
    }
  } else if (kind_ == Kind::Dilu) {
    for (int c = 0; c < nc; ++c) {
      const int64_t b = offsets_[c], e = offsets_[c + 1];
      if (e == b) continue;
      count_launches(1);
#define DC_DILU(B)                                                                                                \
  case B:                                                                                                         \
    k_dilu<B><<<grid_for(e - b), kT, 0, s>>>(b, e, perm_.get(), ipos_.get(), rowptr_, colidx_, diag_, vals,      \
                                             dfac_.get(), status);                                                \
    break;
      switch (bs_) { DC_DILU(1) DC_DILU(2) DC_DILU(3) DC_DILU(4) DC_DILU(5) DC_DILU(6) DC_DILU(7) DC_DILU(8) }
#undef DC_DILU
    }
  }
  // the SELL-32 copy the sweeps read: the ILU(0) factors, else the operator (possibly the
  // caller's)
  const double* src = kind_ == Kind::Ilu0 ? lu_.get() : vals;
  const size_t nv = static_cast<size_t>(sell_.nslots) * 32 * nb2;
  ext_sv32_ = (fp32 && kind_ != Kind::Ilu0 && sell_ext && sv32_ext && sell_ext->nrows == n_ && sell_ext->bs == bs_)
                  ? sv32_ext : nullptr;
  if (ext_sv32_) {
    ext_view_ = *sell_ext;
    sv32_.resize(0);
    if (kind_ == Kind::Dilu) {
      if (dfac32_.size() != dfac_.size()) dfac32_.resize(dfac_.size());
      to_float(static_cast<int64_t>(dfac_.size()), dfac_.get(), dfac32_.get(), s);
    }
  } else if (fp32) {
    if (sv32_.size() != nv) sv32_.resize(nv);
    sell_values(sell_, bs_, src, sv32_.get(), s);
    if (kind_ == Kind::Ilu0 || kind_ == Kind::Dilu) {
      if (dfac32_.size() != dfac_.size()) dfac32_.resize(dfac_.size());
      to_float(static_cast<int64_t>(dfac_.size()), dfac_.get(), dfac32_.get(), s);
    }
  } else {
    if (sv64_.size() != nv) sv64_.resize(nv);
    sell_values(sell_, bs_, src, sv64_.get(), s);
  }
}

template <class T>
void ColorPrecond::sweep_color(int mode, int c, const T* vals, const T* dmat, const T* r, T* z, const double* sc,
                               int done_slot, cudaStream_t s) const {
  using V = T;
  if (offsets_[c + 1] == offsets_[c]) return;
  count_launches(1);
  const Sell S = (ext_sv32_ && std::is_same<T, float>::value) ? ext_view_ : sell_.view(bs_);
  const int gb = grid_for(S.nslices * 32);
  const V w = static_cast<V>(omega);
#define DC_SW(B, M) \
  k_sweep<B, T, M><<<gb, kT, 0, s>>>(S, colour_.get(), c, vals, dmat, r, z, w, sc, done_slot)
#define DC_SWB(B)                                          \
  case B:                                                  \
    switch (mode) {                                        \
      case kSorFirst: DC_SW(B, kSorFirst); break;          \
      case kSorFull: DC_SW(B, kSorFull); break;            \
      case kLowerSolve: DC_SW(B, kLowerSolve); break;      \
      case kUpperSolve: DC_SW(B, kUpperSolve); break;      \
      case kDiluLower: DC_SW(B, kDiluLower); break;        \
      default: DC_SW(B, kDiluUpper); break;                \
    }                                                      \
    break;
  switch (bs_) { DC_SWB(1) DC_SWB(2) DC_SWB(3) DC_SWB(4) DC_SWB(5) DC_SWB(6) DC_SWB(7) DC_SWB(8) }
#undef DC_SWB
#undef DC_SW
}

template <class T>
static const T* pick(const double* d, const float* f) {
  if constexpr (std::is_same<T, float>::value) return f;
  else return d;
}

template <class T>
static void check_precision(bool fp32) {
  if ((std::is_same<T, float>::value) != fp32)
    throw std::runtime_error("multicolour preconditioner: applied in another precision than it was set up for");
}

template <class T>
void ColorPrecond::sor_sweep(const T* r, T* z, bool forward, bool from_zero, const double* sc, int done_slot,
                             cudaStream_t s) const {
  check_precision<T>(fp32_);
  const T* A = pick<T>(sv64_.get(), ext_sv32_ ? ext_sv32_ : sv32_.get());
  const T* D = pick<T>(dinv_, dinv32_);
  if (A == nullptr || D == nullptr) throw std::runtime_error("multicolour sweep: values not set up");
  const int nc = colors();
  if (forward)
    for (int c = 0; c < nc; ++c) sweep_color<T>(from_zero ? kSorFirst : kSorFull, c, A, D, r, z, sc, done_slot, s);
  else
    for (int c = nc - 1; c >= 0; --c) sweep_color<T>(kSorFull, c, A, D, r, z, sc, done_slot, s);
}

template void ColorPrecond::sor_sweep<double>(const double*, double*, bool, bool, const double*, int,
                                              cudaStream_t) const;
template void ColorPrecond::sor_sweep<float>(const float*, float*, bool, bool, const double*, int,
                                             cudaStream_t) const;

template <class T>
void ColorPrecond::apply_t(const T* r, T* z, const double* sc, int done_slot, cudaStream_t s) const {
  check_precision<T>(fp32_);
  const T* A = pick<T>(sv64_.get(), ext_sv32_ ? ext_sv32_ : sv32_.get());  // operator, or the ILU(0) factors
  const T* DF = pick<T>(dfac_.get(), dfac32_.get());
  if (A == nullptr) throw std::runtime_error("multicolour preconditioner: values not set up");
  const int nc = colors();
  switch (kind_) {
    case Kind::Ssor:
    case Kind::Sor:
      for (int it = 0; it < iterations; ++it) {
        sor_sweep<T>(r, z, true, it == 0, sc, done_slot, s);
        if (kind_ == Kind::Ssor) sor_sweep<T>(r, z, false, false, sc, done_slot, s);
      }
      break;
    case Kind::Ilu0:
      for (int c = 0; c < nc; ++c) sweep_color<T>(kLowerSolve, c, A, DF, r, z, sc, done_slot, s);
      for (int c = nc - 1; c >= 0; --c) sweep_color<T>(kUpperSolve, c, A, DF, r, z, sc, done_slot, s);
      break;
    case Kind::Dilu:
      for (int c = 0; c < nc; ++c) sweep_color<T>(kDiluLower, c, A, DF, r, z, sc, done_slot, s);
      for (int c = nc - 1; c >= 0; --c) sweep_color<T>(kDiluUpper, c, A, DF, r, z, sc, done_slot, s);
      break;
  }
}

std::string ColorPrecond::describe() const {
  static const char* names[] = {"SSOR", "SOR", "ILU0", "DILU"};
  return "{\"type\": \"" + std::string(names[static_cast<int>(kind_)]) + "\", \"colours\": " +
         std::to_string(colors()) + ", \"relaxation\": " + std::to_string(omega) +
         ", \"iterations\": " + std::to_string(iterations) + "}";
}

void ColorPrecond::apply(const double* r, double* z, const double* sc, int done_slot, cudaStream_t s) const {
  apply_t<double>(r, z, sc, done_slot, s);
}
void ColorPrecond::apply(const float* r, float* z, const double* sc, int done_slot, cudaStream_t s) const {
  apply_t<float>(r, z, sc, done_slot, s);
}

void RichardsonPrecond::apply(const double* r, double* z, const double* sc, int done_slot, cudaStream_t s) const {
  count_launches(1);
  k_scale<double><<<grid_for(n), kT, 0, s>>>(n, r, z, omega, sc, done_slot);
}
void RichardsonPrecond::apply(const float* r, float* z, const double* sc, int done_slot, cudaStream_t s) const {
  count_launches(1);
  k_scale<float><<<grid_for(n), kT, 0, s>>>(n, r, z, omega, sc, done_slot);
}

}  // namespace dcgpu
