// Shared device/host helpers for the lbm_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/lbm_gb300.h"

#define LBM_HD __host__ __device__ __forceinline__
#define LBM_D __device__ __forceinline__

namespace lbm {

// x / d by a multiply-high with m = ceil(2^32 / d): exact for 0 <= x < 2^32 / d
// (the error x (m d - 2^32) / 2^32 stays below 1 / d there).
struct FastDiv {
  unsigned m;
  int d;
  LBM_D explicit FastDiv(int dv) : m((unsigned)((0x100000000ull + dv - 1) / dv)), d(dv) {}
  LBM_D int div(int x) const { return d == 1 ? x : (int)__umulhi((unsigned)x, m); }
};

// Complex numbers as (re, im) pairs of the working precision.
template <typename R> struct C2 { R x, y; };

template <typename R> LBM_HD C2<R> cmk(R a, R b) { C2<R> c; c.x = a; c.y = b; return c; }
template <typename R> LBM_HD C2<R> operator+(C2<R> a, C2<R> b) { return cmk(a.x + b.x, a.y + b.y); }
template <typename R> LBM_HD C2<R> operator-(C2<R> a, C2<R> b) { return cmk(a.x - b.x, a.y - b.y); }
template <typename R> LBM_HD C2<R> operator*(C2<R> a, R s) { return cmk(a.x * s, a.y * s); }
template <typename R> LBM_HD C2<R> cmul(C2<R> a, C2<R> b) {
  return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R> LBM_HD C2<R> conj(C2<R> a) { return cmk(a.x, -a.y); }
// multiply by +i (SIGN=+1) or -i (SIGN=-1)
template <int SIGN, typename R> LBM_HD C2<R> mul_i(C2<R> a) {
  return SIGN > 0 ? cmk(-a.y, a.x) : cmk(a.y, -a.x);
}
// i*m*a for an integer wavenumber m
template <typename R> LBM_HD C2<R> im_mul(C2<R> a, R m) { return cmk(-a.y * m, a.x * m); }
template <typename R> LBM_HD void cfma(C2<R>& acc, R t, C2<R> v) {
  acc.x = fma(t, v.x, acc.x);
  acc.y = fma(t, v.y, acc.y);
}

// Extended precision for sums that cancel: an unevaluated float pair hi + lo
// built from error-free transformations (Knuth's TwoSum, the FMA form of
// Dekker's TwoProduct) in FP32 mode; plain double in FP64 mode, where the
// working precision already suffices.
template <typename R> struct XF { R hi, lo; };
template <typename R> LBM_HD XF<R> xf(R a) { return {a, R(0)}; }
template <typename R> LBM_HD XF<R> xf_norm(R s, R e) {   // |s| >= |e|
  const R h = s + e;
  return {h, e - (h - s)};
}
template <typename R> LBM_HD XF<R> xf_add(XF<R> a, XF<R> b) {
  if constexpr (sizeof(R) == 8) {
    return {a.hi + b.hi, R(0)};
  } else {
    const R s = a.hi + b.hi, bb = s - a.hi;
    const R e = (a.hi - (s - bb)) + (b.hi - bb);
    return xf_norm(s, e + (a.lo + b.lo));
  }
}
template <typename R> LBM_HD XF<R> xf_prod(R a, R b) {   // a b without rounding
  if constexpr (sizeof(R) == 8) {
    return {a * b, R(0)};
  } else {
    const R p = a * b;
    return {p, fma(a, b, -p)};
  }
}
template <typename R> LBM_HD XF<R> xf_mul(XF<R> a, R b) {
  if constexpr (sizeof(R) == 8) {
    return {a.hi * b, R(0)};
  } else {
    const R p = a.hi * b;
    return xf_norm(p, fma(a.hi, b, -p) + a.lo * b);
  }
}
template <typename R> LBM_HD XF<R> xf_neg(XF<R> a) { return {-a.hi, -a.lo}; }
template <typename R> LBM_HD R xf_val(XF<R> a) { return a.hi + a.lo; }
// complex pairs of XF
template <typename R> struct CX { XF<R> x, y; };
template <typename R> LBM_HD CX<R> cx(C2<R> a) { return {xf(a.x), xf(a.y)}; }
template <typename R> LBM_HD CX<R> cx_add(CX<R> a, CX<R> b) {
  return {xf_add(a.x, b.x), xf_add(a.y, b.y)};
}
template <typename R> LBM_HD CX<R> cx_prod(R s, C2<R> v) { return {xf_prod(s, v.x), xf_prod(s, v.y)}; }
template <typename R> LBM_HD CX<R> cx_mul(CX<R> a, R s) { return {xf_mul(a.x, s), xf_mul(a.y, s)}; }
template <typename R> LBM_HD CX<R> cx_neg(CX<R> a) { return {xf_neg(a.x), xf_neg(a.y)}; }
template <typename R> LBM_HD C2<R> cx_val(CX<R> a) { return cmk(xf_val(a.x), xf_val(a.y)); }

template <typename R> struct Prec;
template <> struct Prec<float> { static constexpr int id = LBM_F32; };
template <> struct Prec<double> { static constexpr int id = LBM_F64; };

// Packed triangular spectral index: rows (m, n) with n = m..N, m-major.
LBM_HD int spec_offset(int m, int N) { return m * (N + 1) - (m * (m - 1)) / 2; }
LBM_HD int spec_index(int m, int n, int N) { return spec_offset(m, N) + (n - m); }
LBM_HD int nspec(int N) { return (N + 1) * (N + 2) / 2; }

template <typename R> LBM_D R ld(const R* p) { return __ldg(p); }

}  // namespace lbm

// Launch-error check shared by the C-ABI entry points.
#define LBM_LAUNCH_CHECK()                                      \
  do {                                                          \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) return LBM_ERR_LAUNCH;               \
  } while (0)
