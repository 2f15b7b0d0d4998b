// Table lookups of the parser context, shared by the host evaluator and the device
// interpreter so that both compute the same bits:
//
//   * interpolation tables (src/dune/copasi/parser/context.cc:68-92): lower_bound over the
//     sorted domain, the first / last range value outside it, std::lerp in between;
//   * functions tabulated with `interpolate = true` (context.cc:237-280);
//   * grayscale TIFF images evaluated at a position (context.cc:62-67,
//     src/dune/copasi/common/tiff_grayscale.cc:94-108).
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define DC_HD __host__ __device__ __forceinline__
#else
#define DC_HD inline
#endif

namespace dcgpu {

// One tabulated function: g[0..intervals] = f(d0 + i (d1 - d0) / intervals).
struct FnTableDesc {
  double d0 = 0.0, d1 = 1.0, ctn = 1.0;  // domain and intervals / (d1 - d0)
  int64_t off = 0;                        // first value in the packed value array
  uint32_t intervals = 1;
  int32_t clamp = 0;                      // out_of_bounds = clamp (1) or error (0)
};

// One grayscale image: pixel (scanline r, column c) at px[off + r * cols + c], already scaled
// to [0, 1] the way the reference scales it.
struct ImageDesc {
  int64_t off = 0;
  uint32_t rows = 0, cols = 0;            // scanlines (ImageLength), samples per scanline (ImageWidth)
  float x_res = 0.f, y_res = 0.f, x_off = 0.f, y_off = 0.f;
};

// std::lerp (C++20, the monotonic / exact-at-ends algorithm of proposal P0811R3): exact when
// a and b straddle zero, b at t == 1, and never past b on the way there.
DC_HD double lerp_exact(double a, double b, double t) {
#ifdef __CUDA_ARCH__
  if ((a <= 0.0 && b >= 0.0) || (a >= 0.0 && b <= 0.0))
    return __dadd_rn(__dmul_rn(t, b), __dmul_rn(__dsub_rn(1.0, t), a));
  if (t == 1.0) return b;
  const double x = __dadd_rn(a, __dmul_rn(t, __dsub_rn(b, a)));
#else
  if ((a <= 0.0 && b >= 0.0) || (a >= 0.0 && b <= 0.0)) return t * b + (1.0 - t) * a;
  if (t == 1.0) return b;
  const double x = a + t * (b - a);
#endif
  return (t > 1.0) == (b > a) ? (b < x ? x : b) : (b > x ? x : b);
}

// interpolation table: X sorted ascending, n >= 2
DC_HD double interp_lookup(const double* X, const double* Y, int n, double x) {
  // std::lower_bound: the first X[d] that is not less than x
  if (!(X[0] < x)) return Y[0];        // x <= X[0] (and NaN, for which no X is less)
  if (X[n - 1] < x) return Y[n - 1];   // past the end
  int lo = 0, hi = n - 1;              // X[lo] < x <= X[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (X[mid] < x) lo = mid; else hi = mid;
  }
#ifdef __CUDA_ARCH__
  const double t = __ddiv_rn(__dsub_rn(x, X[lo]), __dsub_rn(X[hi], X[lo]));
#else
  const double t = (x - X[lo]) / (X[hi] - X[lo]);
#endif
  return lerp_exact(Y[lo], Y[hi], t);
}

// tabulated function.  The reference's lookup blends g[i] with g[j] where both indices are
// the integer part of (x - d0) * ctn, so the result is g[floor((x - d0) * ctn)] exactly (a
// left-endpoint step function), which is what is returned here.  out_of_bounds = clamp
// clamps x into [d0, d1] (NaN to d0); out_of_bounds = error makes an argument outside
// [d0, d1] (or NaN) a NaN, which fails the Newton step.
DC_HD double ftab_lookup(const FnTableDesc& d, const double* g, double x) {
  if (d.clamp) {
    x = (x > d.d0) ? x : d.d0;   // std::max(d0, x): NaN -> d0
    x = (d.d1 < x) ? d.d1 : x;   // std::min(..., d1)
  } else if (!(x >= d.d0 && x <= d.d1)) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(0x7ff8000000000000LL);
#else
    return __builtin_nan("");
#endif
  }
#ifdef __CUDA_ARCH__
  const double pos = __dmul_rn(__dsub_rn(x, d.d0), d.ctn);
#else
  const double pos = (x - d.d0) * d.ctn;
#endif
  uint32_t i = static_cast<uint32_t>(pos);   // pos >= 0: truncation is the integer part
  if (i > d.intervals) i = d.intervals;      // (x - d0) * ctn rounded above the last point
  return g[d.off + i];
}

// float -> uint32 the way the reference's x86-64 build converts: truncate towards zero to a
// 64-bit integer and keep the low 32 bits (0 for NaN and out-of-range values)
DC_HD uint32_t float_to_u32_x86(float v) {
  if (!(v > -9.2e18f && v < 9.2e18f)) return 0u;
  return static_cast<uint32_t>(static_cast<uint64_t>(static_cast<int64_t>(v)));
}

// grayscale image at (x, y): column from x, scanline from y counted from the bottom, both
// clamped to the image (tiff_grayscale.cc:94-108, single-precision arithmetic as there)
DC_HD double image_lookup(const ImageDesc& d, const double* px, double x, double y) {
#ifdef __CUDA_ARCH__
  const float fx = __fmul_rn(d.x_res, __fsub_rn(__double2float_rn(x), d.x_off));
  const float fy = __fmul_rn(d.y_res, __fsub_rn(__double2float_rn(y), d.y_off));
#else
  const float fx = d.x_res * (static_cast<float>(x) - d.x_off);
  const float fy = d.y_res * (static_cast<float>(y) - d.y_off);
#endif
  uint32_t col = float_to_u32_x86(fx);
  uint32_t row = d.rows - float_to_u32_x86(fy) - 1u;   // unsigned wrap-around, as there
  if (col > d.cols - 1u) col = d.cols - 1u;
  if (row > d.rows - 1u) row = d.rows - 1u;
  return px[d.off + static_cast<int64_t>(row) * d.cols + col];
}

}  // namespace dcgpu
