// Real longitude FFT for the spectral transform (I = 64, 128, 256 points).
//
// A real transform of length I = 2L is computed as one complex transform of
// length L (even samples in the real part, odd samples in the imaginary part)
// plus a pairing pass.  The length-L transform is split as L = R1 * R2: a
// team of R1 threads does R2-point DFTs in registers, multiplies by the
// inter-stage twiddles, exchanges through a padded shared-memory tile, then
// does R1-point DFTs.  Teams never span a warp (R1 divides 32), so the only
// synchronisation is __syncwarp on the team mask.
//
// Conventions match the reference (spectral.py:159-172): the forward
// transform returns X_m = (1/I) sum_i x_i exp(-2 pi i m i / I) for
// m = 0..M-1; the inverse evaluates x_i = Re X_0 + 2 Re sum_{m>=1} X_m
// exp(+2 pi i m i / I) (numpy irfft of I*X with the imaginary part of X_0
// dropped and no Nyquist term).
#pragma once
#include "lbm_common.cuh"

namespace lbm {

// ---- small DFTs in registers, natural order in and out ----------------------
template <int SIGN, typename R> LBM_D void dft4(C2<R>* v) {
  C2<R> a0 = v[0] + v[2], a1 = v[0] - v[2];
  C2<R> b0 = v[1] + v[3], b1 = mul_i<SIGN>(v[1] - v[3]);
  v[0] = a0 + b0;
  v[2] = a0 - b0;
  v[1] = a1 + b1;
  v[3] = a1 - b1;
}

template <int SIGN, typename R> LBM_D void dft8(C2<R>* v) {
  C2<R> e[4] = {v[0], v[2], v[4], v[6]};
  C2<R> o[4] = {v[1], v[3], v[5], v[7]};
  dft4<SIGN>(e);
  dft4<SIGN>(o);
  const R h = R(0.70710678118654752440);
  // W8^1 = h(1 + SIGN i), W8^2 = SIGN i, W8^3 = h(-1 + SIGN i)
  C2<R> t1 = cmk<R>(h * (o[1].x - SIGN * o[1].y), h * (o[1].y + SIGN * o[1].x));
  C2<R> t2 = mul_i<SIGN>(o[2]);
  C2<R> t3 = cmk<R>(h * (-o[3].x - SIGN * o[3].y), h * (-o[3].y + SIGN * o[3].x));
  v[0] = e[0] + o[0];
  v[4] = e[0] - o[0];
  v[1] = e[1] + t1;
  v[5] = e[1] - t1;
  v[2] = e[2] + t2;
  v[6] = e[2] - t2;
  v[3] = e[3] + t3;
  v[7] = e[3] - t3;
}

template <int SIGN, typename R> LBM_D void dft16(C2<R>* v) {
  C2<R> e[8], o[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    e[i] = v[2 * i];
    o[i] = v[2 * i + 1];
  }
  dft8<SIGN>(e);
  dft8<SIGN>(o);
  // cos/sin(2 pi k / 16), k = 0..7
  const R c[8] = {R(1.0), R(0.92387953251128675613), R(0.70710678118654752440),
                  R(0.38268343236508977173), R(0.0), R(-0.38268343236508977173),
                  R(-0.70710678118654752440), R(-0.92387953251128675613)};
  const R s[8] = {R(0.0), R(0.38268343236508977173), R(0.70710678118654752440),
                  R(0.92387953251128675613), R(1.0), R(0.92387953251128675613),
                  R(0.70710678118654752440), R(0.38268343236508977173)};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    C2<R> w = cmk<R>(c[k], R(SIGN) * s[k]);
    C2<R> t = cmul(w, o[k]);
    v[k] = e[k] + t;
    v[k + 8] = e[k] - t;
  }
}

template <int SIGN, int N, typename R> LBM_D void dft(C2<R>* v) {
  if constexpr (N == 4) dft4<SIGN>(v);
  else if constexpr (N == 8) dft8<SIGN>(v);
  else dft16<SIGN>(v);
}

// ---- decomposition of the half-length complex transform ----------------------
template <int I> struct FftShape;
template <> struct FftShape<64> { static constexpr int R1 = 4, R2 = 8; };
template <> struct FftShape<128> { static constexpr int R1 = 8, R2 = 8; };
template <> struct FftShape<256> { static constexpr int R1 = 8, R2 = 16; };

// Shared-memory scratch (complex elements) one team needs.
template <int I> __host__ __device__ constexpr int fft_team_scratch() {
  return FftShape<I>::R1 * (FftShape<I>::R2 + 1);
}

LBM_D unsigned team_mask(int R1) {
  const int lane = threadIdx.x & 31;
  const unsigned base = (R1 == 32) ? 0xffffffffu : ((1u << R1) - 1u);
  return (R1 == 32) ? base : (base << (lane & ~(R1 - 1)));
}

// Length-L complex DFT over the team; input already in registers as
// v[r] = z[t + R1 r], result z'[s + R2 u] written to scr in natural order.
// tw[p] = exp(-2 pi i p / I), p in [0, I).
template <int SIGN, int I, typename R>
LBM_D void team_cfft(int t, C2<R>* v, C2<R>* scr, const C2<R>* tw, unsigned mask) {
  constexpr int R1 = FftShape<I>::R1, R2 = FftShape<I>::R2, P = R2 + 1;
  dft<SIGN, R2>(v);
#pragma unroll
  for (int s = 1; s < R2; ++s) {
    C2<R> w = tw[2 * t * s];
    if (SIGN > 0) w.y = -w.y;
    v[s] = cmul(v[s], w);
  }
#pragma unroll
  for (int s = 0; s < R2; ++s) scr[t * P + s] = v[s];
  __syncwarp(mask);
  constexpr int NC = R2 / R1;
  C2<R> w[NC][R1];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int s = t + R1 * c;
#pragma unroll
    for (int u = 0; u < R1; ++u) w[c][u] = scr[u * P + s];
  }
  __syncwarp(mask);
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    dft<SIGN, R1>(w[c]);
    const int s = t + R1 * c;
#pragma unroll
    for (int u = 0; u < R1; ++u) scr[s + R2 * u] = w[c][u];
  }
  __syncwarp(mask);
}

// Forward real FFT of x[i * xs], i < I, by the team; calls out(m, X_m) for
// m < M with X_m already scaled by `scale` (normally 1/I times a weight).
template <int I, typename R, typename Out>
LBM_D void team_rfft_fwd(int t, const R* x, int xs, C2<R>* scr, const C2<R>* tw, int M,
                         R scale, Out out) {
  constexpr int R1 = FftShape<I>::R1, R2 = FftShape<I>::R2, L = I / 2;
  const unsigned mask = team_mask(R1);
  C2<R> v[R2];
#pragma unroll
  for (int r = 0; r < R2; ++r) {
    const int n = t + R1 * r;
    v[r] = cmk<R>(x[(2 * n) * xs], x[(2 * n + 1) * xs]);
  }
  team_cfft<-1, I>(t, v, scr, tw, mask);
  for (int m = t; m < M; m += R1) {
    C2<R> zk = scr[m];
    C2<R> zc = conj(scr[(L - m) & (L - 1)]);
    C2<R> ev = (zk + zc) * R(0.5);
    C2<R> od = mul_i<-1>(zk - zc) * R(0.5);
    C2<R> X = ev + cmul(tw[m], od);
    out(m, X * scale);
  }
  __syncwarp(mask);
}

// Inverse real FFT: in(m) supplies X_m for m < M; writes x[i * xs], i < I,
// each value multiplied by `scale`.
template <int I, typename R, typename In>
LBM_D void team_rfft_inv(int t, In in, int M, C2<R>* scr, const C2<R>* tw, R* x, int xs,
                         R scale) {
  constexpr int R1 = FftShape<I>::R1, R2 = FftShape<I>::R2, L = I / 2;
  const unsigned mask = team_mask(R1);
  C2<R> v[R2];
#pragma unroll
  for (int r = 0; r < R2; ++r) {
    const int n = t + R1 * r;
    C2<R> y = cmk<R>(R(0), R(0));
    if (n < M) y = in(n);
    if (n == 0) y.y = R(0);
    C2<R> yc = cmk<R>(R(0), R(0));
    if (n > 0 && L - n < M) yc = conj(in(L - n));
    C2<R> w = conj(tw[n]);
    v[r] = (y + yc) + mul_i<1>(cmul(w, y - yc));
  }
  team_cfft<1, I>(t, v, scr, tw, mask);
  // z_k is at scr[k]; x[2k] = Re z_k, x[2k+1] = Im z_k
  for (int k = t; k < L; k += R1) {
    C2<R> z = scr[k];
    x[(2 * k) * xs] = z.x * scale;
    x[(2 * k + 1) * xs] = z.y * scale;
  }
  __syncwarp(mask);
}

}  // namespace lbm
