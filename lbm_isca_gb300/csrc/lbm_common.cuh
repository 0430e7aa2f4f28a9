// Shared device/host helpers for the lbm_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/lbm_gb300.h"

#define LBM_HD __host__ __device__ __forceinline__
#define LBM_D __device__ __forceinline__

namespace lbm {

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
