// k_grid_dft: the grid-point kernel of the fused stepper for FP32, with the
// longitude transforms as dense DFTs folded by the symmetries of the
// longitude circle and written as register-tiled small GEMMs on CUDA cores.
//
// Inverse (Fourier -> grid), per field, with A_m = 2 Re X_m, B_m = 2 Im X_m
// (A_0 = Re X_0, B_0 = 0) and for i in [1, I/4]:
//   CE = sum_{m even} A_m cos(2 pi m i/I), CO = sum_{m odd} A_m cos(.),
//   SE = sum_{m even} B_m sin(.),          SO = sum_{m odd} B_m sin(.)
//   x_i = CE+CO-SE-SO, x_{I-i} = CE+CO+SE+SO,
//   x_{I/2-i} = CE-CO+SE-SO, x_{I/2+i} = CE-CO-SE+SO;
//   x_0 = sum A_m, x_{I/2} = sum (-1)^m A_m.
// Forward (grid -> Fourier), X_m = (1/I) sum_i x_i exp(-2 pi i m i/I): with
// u_i = x_i + x_{I-i}, v_i = x_i - x_{I-i} and for i in [1, I/4 - 1]
//   ue = u_i + u_{I/2-i}, uo = u_i - u_{I/2-i}, ve = v_i - v_{I/2-i},
//   vo = v_i + v_{I/2-i},
//   I Re X_m = x_0 + (-1)^m x_{I/2} + [m even] (-1)^{m/2} u_{I/4}
//              + sum_i (m even ? ue : uo) cos(2 pi m i/I)
//  -I Im X_m = [m odd] (-1)^{(m-1)/2} v_{I/4} + sum_i (m even ? ve : vo) sin(.)
// ~2.8K FMAs per field at I = 128, against ~11K for the plain dense DFT.
// The table (cos, sin)(2 pi m i / I), m < M, i <= I/4, is computed in FP64
// on the host and rounded once.
//
// Per level batch (KB levels): stage the Fourier inputs, inverse DFTs into a
// ring of grid levels, per-(column, level) contributions to the column
// sums, a per-column scan, the pointwise algebra, folding, forward DFTs
// with the analysis weights, store.
#pragma once

namespace lbm {

// Vertical advection of dynamics.py's _vert_advect written in differences,
//   (s1 (f[k+1] - f[k]) / 2 + s0 (f[k] - f[k-1]) / 2) / dsig_k
// (at the bottom / top the missing half becomes +s0 f[k] / -s1 f[k]), which
// equals the flux form (F[k+1/2] - F[k-1/2] - f[k] (s1 - s0)) / dsig_k with
// F = s (f[k] + f[k+-1]) / 2 without cancelling the f[k] (s1 - s0) part.
// vadv_p: perturbation field; vadv_b: basic state with its half differences
// hm = (f[k] - f[k-1]) / 2, hp = (f[k+1] - f[k]) / 2 precomputed in FP64.
LBM_D float vadv_p(float fm, float f0, float fp, float s0, float s1, bool lo, bool hi,
                   float dsk) {
  const float up = hi ? 0.5f * s1 * (fp - f0) : -s1 * f0;
  const float dn = lo ? 0.5f * s0 * (f0 - fm) : s0 * f0;
  return (up + dn) / dsk;
}
LBM_D float vadv_b(float f0, float hm, float hp, float s0, float s1, bool lo, bool hi,
                   float dsk) {
  const float up = hi ? s1 * hp : -s1 * f0;
  const float dn = lo ? s0 * hm : s0 * f0;
  return (up + dn) / dsk;
}

template <int I> struct DftGrid {
  static constexpr int Q = I / 4;
  static constexpr int NT = 256;
  static constexpr int NW = NT / 32;
  static constexpr int KB = (I == 256) ? 2 : 4;   // levels per batch (SMEM-bound)
  static constexpr int RS = KB + 2;
  static constexpr int NG = 9;
};

// Shared-memory carve-up (float units); every block starts 16-byte aligned.
struct DftLayout {
  int tab, fin, fout, ring, gout, fw, pre, pst, sg, vert, total;
  LBM_HD static int al4(int x) { return (x + 3) & ~3; }
  LBM_HD DftLayout(int I, int M, int K, int KB) {
    const int Q = I / 4;
    int o = 0;
    tab = o; o = al4(o + 2 * M * (Q + 1));
    fin = o; o = al4(o + 2 * 2 * (KB + 1) * 6 * M);   // two buffers [M][(KB+1)*6]
    fout = o; o = al4(o + 2 * KB * 7 * M);
    ring = o; o = al4(o + (KB + 2) * 6 * I);
    gout = o; o = al4(o + KB * 9 * I);
    fw = o; o = al4(o + KB * 9 * (Q + 1) * 4);
    pre = o; o = al4(o + KB * 5 * I);
    pst = o; o = al4(o + 5 * I);
    sg = o; o = al4(o + 8 * I);
    vert = o; o = al4(o + LBM_VERT_COUNT * (K + 1));
    total = o;
  }
};

// Inverse transforms of `nf` fields.  Field f reads its raw Fourier
// coefficients X_m at fin[m * ms + f * fs] (the imaginary part of X_0 is
// ignored, the factor 2 of m >= 1 applied here) and writes x_i through
// store(f, i, value).
template <int I, typename Store>
LBM_D void dft_inverse(const float2* __restrict__ tab, const float2* __restrict__ fin, int ms,
                       int fs, int nf, int M, Store store) {
  constexpr int Q = I / 4, NT = DftGrid<I>::NT;
  const int tid = threadIdx.x;
  const int ntrip = (nf + 2) / 3;
  for (int it = tid; it < Q * ntrip; it += NT) {
    const int i = it % Q + 1, tr = it / Q;
    float ce0 = 0, co0 = 0, se0 = 0, so0 = 0, ce1 = 0, co1 = 0, se1 = 0, so1 = 0;
    float ce2 = 0, co2 = 0, se2 = 0, so2 = 0;
    const int f0 = 3 * tr;
    const float2* x0 = fin + min(f0, nf - 1) * fs;
    const float2* x1 = fin + min(f0 + 1, nf - 1) * fs;
    const float2* x2 = fin + min(f0 + 2, nf - 1) * fs;
    const float2* tb = tab + i;
    int m = 1;
#pragma unroll 3
    for (; m + 1 < M; m += 2) {               // (odd, even) pairs of m >= 1
      const float2 to = tb[m * (Q + 1)], te = tb[(m + 1) * (Q + 1)];
      const float2 b0 = x0[m * ms], a0 = x0[(m + 1) * ms];
      const float2 b1 = x1[m * ms], a1 = x1[(m + 1) * ms];
      const float2 b2 = x2[m * ms], a2 = x2[(m + 1) * ms];
      ce0 = fmaf(a0.x, te.x, ce0); se0 = fmaf(a0.y, te.y, se0);
      co0 = fmaf(b0.x, to.x, co0); so0 = fmaf(b0.y, to.y, so0);
      ce1 = fmaf(a1.x, te.x, ce1); se1 = fmaf(a1.y, te.y, se1);
      co1 = fmaf(b1.x, to.x, co1); so1 = fmaf(b1.y, to.y, so1);
      ce2 = fmaf(a2.x, te.x, ce2); se2 = fmaf(a2.y, te.y, se2);
      co2 = fmaf(b2.x, to.x, co2); so2 = fmaf(b2.y, to.y, so2);
    }
    if (m < M) {                               // last (odd) m
      const float2 to = tb[m * (Q + 1)];
      const float2 b0 = x0[m * ms], b1 = x1[m * ms], b2 = x2[m * ms];
      co0 = fmaf(b0.x, to.x, co0); so0 = fmaf(b0.y, to.y, so0);
      co1 = fmaf(b1.x, to.x, co1); so1 = fmaf(b1.y, to.y, so1);
      co2 = fmaf(b2.x, to.x, co2); so2 = fmaf(b2.y, to.y, so2);
    }
    const float ce[3] = {x0[0].x + 2.f * ce0, x1[0].x + 2.f * ce1, x2[0].x + 2.f * ce2};
    const float co[3] = {2.f * co0, 2.f * co1, 2.f * co2};
    const float se[3] = {2.f * se0, 2.f * se1, 2.f * se2};
    const float so[3] = {2.f * so0, 2.f * so1, 2.f * so2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int f = f0 + q;
      if (f >= nf) break;
      const float p = ce[q] + co[q], mn = ce[q] - co[q];
      const float s = se[q] + so[q], dd = se[q] - so[q];
      store(f, i, p - s);
      store(f, I - i, p + s);
      store(f, I / 2 - i, mn + dd);
      store(f, I / 2 + i, mn - dd);
    }
  }
  // i = 0 and i = I/2: lane-parallel sums per field, one warp per field
  const int lane = tid & 31;
  for (int f = tid >> 5; f < nf; f += NT / 32) {
    const float2* x = fin + f * fs;
    float s0 = 0.f, s1 = 0.f;
    for (int m = 1 + lane; m < M; m += 32) {
      const float a = x[m * ms].x;
      s0 += a;
      s1 += (m & 1) ? -a : a;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if (lane == 0) {
      store(f, 0, x[0].x + 2.f * s0);
      store(f, I / 2, x[0].x + 2.f * s1);
    }
  }
}

// Asynchronous 16-byte global -> shared copies (cp.async, completion groups).
LBM_D void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
LBM_D void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> LBM_D void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Fold nf grid fields (field f at base + f * I) into fw[f][i][4].
template <int I>
LBM_D void dft_fold(float4* __restrict__ fw, int nf, const float* __restrict__ base) {
  constexpr int Q = I / 4, NT = DftGrid<I>::NT;
  for (int it = threadIdx.x; it < nf * (Q + 1); it += NT) {
    const int f = it / (Q + 1), i = it - f * (Q + 1);
    const float* x = base + f * I;
    float4 r;
    if (i == 0) {
      const float xq = x[Q], x3q = x[3 * Q];
      r = make_float4(x[0], x[I / 2], xq + x3q, xq - x3q);
    } else if (i == Q) {
      r = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      const float xa = x[i], xb = x[I - i], xc = x[I / 2 - i], xd = x[I / 2 + i];
      const float u = xa + xb, v = xa - xb, uh = xc + xd, vh = xc - xd;
      r = make_float4(u + uh, u - uh, v - vh, v + vh);
    }
    fw[it] = r;
  }
}

// Forward transforms of the folded fields, 4 per thread item; quad(q, k)
// returns the folded-field index of member k (0..3) of quad q (or -1), and
// emit(q, m, fi, X[4]) receives I * X_m of the quad's fields.
template <int I, typename Quad, typename Emit>
LBM_D void dft_forward(const float2* __restrict__ tab, const float4* __restrict__ fw, int nquad,
                       int M, Quad quad, Emit emit) {
  constexpr int Q = I / 4, NT = DftGrid<I>::NT;
  const int NPm = (M + 1) / 2;
  for (int it = threadIdx.x; it < NPm * nquad; it += NT) {
    const int q = it / NPm, p = it - q * NPm;
    const int me = 2 * p, mo = 2 * p + 1;
    const bool hmo = mo < M;
    int fi[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) fi[k] = quad(q, k);
    float re_e[4] = {0, 0, 0, 0}, im_e[4] = {0, 0, 0, 0}, re_o[4] = {0, 0, 0, 0},
          im_o[4] = {0, 0, 0, 0};
    const float2* te_row = tab + me * (Q + 1);
    const float2* to_row = tab + (hmo ? mo : me) * (Q + 1);
    const float4* w0 = fw + (fi[0] >= 0 ? fi[0] : 0) * (Q + 1);
    const float4* w1 = fw + (fi[1] >= 0 ? fi[1] : 0) * (Q + 1);
    const float4* w2 = fw + (fi[2] >= 0 ? fi[2] : 0) * (Q + 1);
    const float4* w3 = fw + (fi[3] >= 0 ? fi[3] : 0) * (Q + 1);
#pragma unroll 5
    for (int i = 1; i < Q; ++i) {
      const float2 te = te_row[i], to = to_row[i];
      const float4 a = w0[i], b = w1[i], c = w2[i], e = w3[i];
      re_e[0] = fmaf(a.x, te.x, re_e[0]); im_e[0] = fmaf(a.z, te.y, im_e[0]);
      re_o[0] = fmaf(a.y, to.x, re_o[0]); im_o[0] = fmaf(a.w, to.y, im_o[0]);
      re_e[1] = fmaf(b.x, te.x, re_e[1]); im_e[1] = fmaf(b.z, te.y, im_e[1]);
      re_o[1] = fmaf(b.y, to.x, re_o[1]); im_o[1] = fmaf(b.w, to.y, im_o[1]);
      re_e[2] = fmaf(c.x, te.x, re_e[2]); im_e[2] = fmaf(c.z, te.y, im_e[2]);
      re_o[2] = fmaf(c.y, to.x, re_o[2]); im_o[2] = fmaf(c.w, to.y, im_o[2]);
      re_e[3] = fmaf(e.x, te.x, re_e[3]); im_e[3] = fmaf(e.z, te.y, im_e[3]);
      re_o[3] = fmaf(e.y, to.x, re_o[3]); im_o[3] = fmaf(e.w, to.y, im_o[3]);
    }
    // boundary terms: (x0, x_{I/2}, u_{I/4}, v_{I/4}) in slot 0
    const float ce = (p & 1) ? -1.f : 1.f;            // (-1)^{me/2}
    const float so = (((mo - 1) / 2) & 1) ? -1.f : 1.f;  // (-1)^{(mo-1)/2}
    const float4* ws[4] = {w0, w1, w2, w3};
    float2 Xe[4], Xo[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 b0 = ws[k][0];
      Xe[k] = make_float2(re_e[k] + b0.x + b0.y + ce * b0.z, -im_e[k]);
      Xo[k] = make_float2(re_o[k] + b0.x - b0.y, -(im_o[k] + so * b0.w));
    }
    emit(q, me, fi, Xe);
    if (hmo) emit(q, mo, fi, Xo);
  }
}

// ---------------------------------------------------------------------------
template <int I>
__global__ void __launch_bounds__(DftGrid<I>::NT) k_grid_dft(SD<float> d, const float2* dft,
                                                            int ps_mode) {
  using G = DftGrid<I>;
  constexpr int Q = G::Q, NT = G::NT, NW = G::NW, KB = G::KB, RS = G::RS, NG = G::NG;
  const int j = blockIdx.x, e = blockIdx.y;
  const int J = d.J, K = d.K, M = d.M;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const DftLayout L(I, M, K, KB);
  extern __shared__ float4 sm4[];
  float* sm = reinterpret_cast<float*>(sm4);
  float2* tab = reinterpret_cast<float2*>(sm + L.tab);
  float2* fin = reinterpret_cast<float2*>(sm + L.fin);
  float2* fout = reinterpret_cast<float2*>(sm + L.fout);
  float* ring = sm + L.ring;          // [RS][6][I]
  float* gout = sm + L.gout;          // [KB][9][I]
  float4* fw = reinterpret_cast<float4*>(sm + L.fw);   // [KB*9][Q+1]
  float* pre = sm + L.pre;            // [KB][5][I]
  float* pst = sm + L.pst;            // [5][I]
  float* sg = sm + L.sg;              // [8][I]
  float* vert = sm + L.vert;          // [VERT][K+1]

  for (int x = tid; x < M * (Q + 1); x += NT) tab[x] = dft[x];
  for (int x = tid; x < LBM_VERT_COUNT * (K + 1); x += NT) vert[x] = d.vert[x];
  for (int x = tid; x < 5 * I; x += NT) pst[x] = 0.f;
  auto V = [&](int row, int k) { return vert[row * (K + 1) + k]; };
  const float gw = d.jfac[JF_GW * J + j], gwdc = d.jfac[JF_GWDELC * J + j];
  const float rcos = d.jfac[JF_RCOS * J + j];
  const float wg = gw / float(I), wd = gwdc / float(I);
  const size_t jmK = (size_t)J * K;
  const float2* sfe = reinterpret_cast<const float2*>(d.sf) + (size_t)e * M * jmK * SF_N;
  float2* afe = reinterpret_cast<float2*>(d.af) + (size_t)e * M * jmK * AF_N;
  const float* b2 = d.b2;
  // basic state of this latitude: field f, level k, column c
  const float* b3j = d.b3 + (size_t)j * K * I;
  const size_t b3f = (size_t)J * K * I;
  auto B3 = [&](int f, int k, int c) -> float { return __ldg(b3j + f * b3f + k * I + c); };

  // Fourier rows of one level batch: levels lo..lo+nl-1, 6 fields, per m a
  // contiguous run of nl*6 complex values -> fbuf[b][m][0 .. nl*6)
  constexpr int RW = (KB + 1) * SF_N;
  auto fbuf = [&](int b) { return fin + (size_t)b * M * RW; };
  auto batch_range = [&](int k0, int& lo, int& nl) {
    lo = (k0 == 0) ? 0 : k0 + 1;
    nl = min(k0 + KB, K - 1) - lo + 1;
  };
  auto prefetch = [&](int k0, float2* buf) {
    int lo, nl;
    batch_range(k0, lo, nl);
    const int chunks = nl * SF_N / 2;          // 16-byte chunks per m-row
    if (nl > 0)
      for (int m = warp; m < M; m += NW)
        for (int c = lane; c < chunks; c += 32)
          cp_async16(buf + (size_t)m * RW + 2 * c,
                     sfe + ((size_t)m * J + j) * K * SF_N + (size_t)lo * SF_N + 2 * c);
    cp_async_commit();
  };
  prefetch(0, fbuf(0));

  // ---- surface pre-pass --------------------------------------------------------
  // fields: 0 pi, 1 pi_x = i m pi / (a cos), 2 pi_y, 3 U-sum, 4 V-sum, 5 D-sum
  float2* fs0 = fbuf(1);
  for (int x = tid; x < M * SFS_N; x += NT) {
    const int m = x / SFS_N, f = x - m * SFS_N;
    const float2 X = reinterpret_cast<const float2*>(d.sfs)[(((size_t)e * M + m) * J + j) * SFS_N + f];
    if (f == SFS_PI) {
      fs0[0 * M + m] = X;
      fs0[1 * M + m] = make_float2(-X.y * m * rcos, X.x * m * rcos);
    } else {
      const float s = (f == SFS_DH) ? 1.f : rcos;
      fs0[(f + 1) * M + m] = make_float2(X.x * s, X.y * s);
    }
  }
  __syncthreads();
  dft_inverse<I>(tab, fs0, 1, M, 6, M, [&](int f, int i, float x) { sg[f * I + i] = x; });
  __syncthreads();
  for (int c = tid; c < I; c += NT) {
    const size_t g2 = (size_t)j * I + c;
    const float pixb = b2[(B2_PIX * J) * I + g2], piyb = b2[(B2_PIY * J) * I + g2];
    const float psbar = b2[(B2_PSBAR * J) * I + g2];
    const float usum = b2[(B2_USUM * J) * I + g2], vsum = b2[(B2_VSUM * J) * I + g2];
    const float pi = sg[0 * I + c], pix = sg[1 * I + c], piy = sg[2 * I + c];
    const float uh = sg[3 * I + c], vh = sg[4 * I + c], dh = sg[5 * I + c];
    const float sx = pixb * uh + piyb * vh + pix * usum + piy * vsum;
    sg[3 * I + c] = pixb;                        // (slots 3, 4 reused: basic grad ln ps)
    sg[4 * I + c] = piyb;
    sg[5 * I + c] = sx;                          // sum_k dsig v.grad(pi)
    sg[6 * I + c] = dh + sx;                     // S_tot
    sg[7 * I + c] = dh;
    // sigma-dot at the lowest interface, (sigm_0 - 1) S_tot
    pst[c] = (V(LBM_VERT_SIGM, 0) - 1.f) * (dh + sx);
    gout[0 * I + c] = -sx;                       // gt_pi = -sum dsig v.grad(pi)
    const size_t gp = (size_t)e * J * I + g2;
    const float pscur = psbar * expm1f(pi);
    float pb = d.psb[gp];
    if (ps_mode == 1) {
      pb = d.psa[gp];
    } else if (ps_mode == 2) {
      const float pa = d.psa[gp];
      pb = pa + d.robert * (pb - 2.f * pa + pscur);
    }
    if (ps_mode != 0) {
      d.psb[gp] = pb;
      d.psa[gp] = pscur;
    }
    gout[1 * I + c] = log1pf(pb / psbar);
  }
  __syncthreads();
  dft_fold<I>(fw, 2, gout);
  __syncthreads();
  dft_forward<I>(tab, fw, 1, M, [](int q, int k) { return k < 2 ? k : -1; },
                 [&](int q, int m, const int* fi, const float2* X) {
                   float2* o = reinterpret_cast<float2*>(d.afs) + (((size_t)e * M + m) * J + j) * 2;
                   o[0] = make_float2(X[0].x * wg, X[0].y * wg);
                   o[1] = make_float2(X[1].x * wg, X[1].y * wg);
                 });

  // ---- level loop -------------------------------------------------------------
  const float eps = d.epsvt, kappa = d.kappa;
  auto RG = [&](int k, int f) -> float* { return ring + ((k % RS) * SF_N + f) * I; };
  int bsel = 0;
  for (int k0 = 0; k0 < K; k0 += KB) {
    int lo, nl;
    batch_range(k0, lo, nl);
    const int kb = min(KB, K - k0);
    __syncthreads();
    // the next batch's rows stream in while this batch computes
    if (k0 + KB < K) prefetch(k0 + KB, fbuf(bsel ^ 1));
    else cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    if (nl > 0) {
      dft_inverse<I>(tab, fbuf(bsel), RW, 1, nl * SF_N, M, [&](int f, int i, float x) {
        const int l = f / SF_N, fld = f - l * SF_N;
        RG(lo + l, fld)[i] = (fld == SF_U || fld == SF_V) ? x * rcos : x;
      });
      __syncthreads();
    }
    bsel ^= 1;
    // contributions to the column sums, one (level, column) per item
    for (int it = tid; it < kb * I; it += NT) {
      const int l = it / I, c = it - l * I, k = k0 + l;
      const float pix = sg[1 * I + c], piy = sg[2 * I + c];
      const float pixb = sg[3 * I + c], piyb = sg[4 * I + c];
      const float uu = RG(k, SF_U)[c], vv = RG(k, SF_V)[c], dd = RG(k, SF_DIV)[c];
      const float tt = RG(k, SF_T)[c], qq = RG(k, SF_Q)[c];
      const float pa = uu * pixb + B3(B_U, k, c) * pix + vv * piyb + B3(B_V, k, c) * piy;
      float* pr = pre + (l * 5) * I;
      pr[0 * I + c] = (dd + pa - sg[6 * I + c]) * V(LBM_VERT_DSIG, k);
      pr[1 * I + c] = dd * V(LBM_VERT_DSIG, k);
      pr[2 * I + c] = eps * (tt * B3(B_Q, k, c) + B3(B_T, k, c) * qq);   // Tv' - T'
      pr[3 * I + c] = pa;
    }
    __syncthreads();
    // per-column scan over the batch's levels.  sigma-dot runs as the sum of
    // dsig (D + v.grad(pi) - S_tot) (no total-minus-prefix cancellation); the
    // suffix sums of dsig D and of dsig v.grad(pi) are kept apart so that the
    // temperature equation can cancel its reference-temperature part exactly
    for (int c = tid; c < I; c += NT) {
      const float dh = sg[7 * I + c], ptot = sg[5 * I + c];
      float sdot = pst[c], prefd = pst[I + c], pref3 = pst[2 * I + c], prefp = pst[3 * I + c];
      pst[4 * I + c] = sdot;                                       // lower interface of lo
      for (int l = 0; l < kb; ++l) {
        const int k = k0 + l;
        float* pr = pre + (l * 5) * I;
        const float cc = pr[0 * I + c], cd = pr[1 * I + c], x = pr[2 * I + c];
        const float pa = pr[3 * I + c];
        pr[4 * I + c] = pref3 + V(LBM_VERT_RALPHA, k) * x;        // (WW (Tv'-T'))_k
        sdot += cc;
        pr[0 * I + c] = sdot;                                      // sigma-dot at k+1/2
        prefd += cd;
        pr[2 * I + c] = dh - prefd;                                // sum_{l>k} dsig div
        prefp += V(LBM_VERT_DSIG, k) * pa;
        pr[1 * I + c] = ptot - prefp;                              // sum_{l>k} dsig v.grad(pi)
        pref3 += V(LBM_VERT_RDLOG3, k) * x;
      }
      pst[c] = sdot;
      pst[I + c] = prefd;
      pst[2 * I + c] = pref3;
      pst[3 * I + c] = prefp;
    }
    __syncthreads();
    // pointwise algebra, (level, column) per item
    for (int it = tid; it < kb * I; it += NT) {
      const int l = it / I, c = it - l * I, k = k0 + l;
      const bool hasm = k >= 1, hasp = k + 1 <= K - 1;
      // basic state at k (and k-1, k+1): all global loads issued first
      const float* bk = b3j + (size_t)k * I + c;
      const int om = hasm ? -I : 0;
      const float ub = __ldg(bk + B_U * b3f), vb = __ldg(bk + B_V * b3f);
      const float tb = __ldg(bk + B_T * b3f), qb = __ldg(bk + B_Q * b3f);
      const float tvb = __ldg(bk + B_TV * b3f), absv = __ldg(bk + B_ABSVOR * b3f);
      const float divb = __ldg(bk + B_DIV * b3f), x5b = __ldg(bk + B_X5 * b3f);
      const float tdev = __ldg(bk + B_TDEV * b3f), tvdev = __ldg(bk + B_TVDEV * b3f);
      // half vertical differences 0.5 (f[k+1] - f[k]) of ub, vb, tb, qb at k-1 and k
      const float hum = __ldg(bk + B_HDU * b3f + om), hup = __ldg(bk + B_HDU * b3f);
      const float hvm = __ldg(bk + B_HDV * b3f + om), hvp = __ldg(bk + B_HDV * b3f);
      const float htm = __ldg(bk + B_HDT * b3f + om), htp = __ldg(bk + B_HDT * b3f);
      const float hqm = __ldg(bk + B_HDQ * b3f + om), hqp = __ldg(bk + B_HDQ * b3f);
      const float* bsdk = d.bsd + ((size_t)j * (K + 1) + k) * I + c;
      const float sb0 = __ldg(bsdk), sb1 = __ldg(bsdk + I);
      const float pix = sg[1 * I + c], piy = sg[2 * I + c];
      const float pixb = sg[3 * I + c], piyb = sg[4 * I + c];
      const float* pr = pre + (l * 5) * I;
      const float sdv = pr[2 * I + c], spv = pr[1 * I + c];
      const float padv = pr[3 * I + c], phiv = pr[4 * I + c];
      const float* vk = vert + k;              // per-level constants at row * (K+1)
      const int VS = K + 1;
      // sigma-dot at the lower (k-1/2) and upper (k+1/2) interfaces
      const float sd0 = hasm ? (l > 0 ? pre[((l - 1) * 5) * I + c] : pst[4 * I + c]) : 0.f;
      const float sd1 = hasp ? pr[0 * I + c] : 0.f;
      const float dsk = vk[LBM_VERT_DSIG * VS];
      const float* r0 = ring + ((k % RS) * SF_N) * I + c;
      const float* rm = ring + (((hasm ? k - 1 : k) % RS) * SF_N) * I + c;
      const float* rp = ring + (((hasp ? k + 1 : k) % RS) * SF_N) * I + c;
      const float u = r0[SF_U * I], v = r0[SF_V * I], vo = r0[SF_VOR * I];
      const float dv = r0[SF_DIV * I], tt = r0[SF_T * I], q = r0[SF_Q * I];
      const float tv = tt + eps * (tt * qb + tb * q);
      const float al = vk[LBM_VERT_ALPHA * VS], w3 = vk[LBM_VERT_W3 * VS];
      // adiabatic term plus the reference-temperature matrix, with Tref
      // cancelled algebraically: -kappa (Tv' x5b + Tvb x5') + kappa Tref
      // (alpha D + w3 sum_{l>k} dsig D)
      const float adtm = -kappa * (tv * x5b + tvdev * (al * dv + w3 * sdv) +
                                   tvb * (vk[LBM_VERT_WP * VS] * padv + w3 * spv));
      const float hadv = tt * divb + tdev * dv;
      const float vadvT = vadv_p(rm[SF_T * I], tt, rp[SF_T * I], sb0, sb1, hasm, hasp, dsk) +
                          vadv_b(tb, htm, htp, sd0, sd1, hasm, hasp, dsk);
      float* go = gout + (l * NG) * I + c;
      // field order per level: 0 gt 1 xu 2 g 3 yu | 4 fu 5 fv 6 ke 7 xv | 8 yv
      go[0 * I] = adtm + hadv + vadvT;
      go[1 * I] = u * tdev + ub * tt;
      const float rcpg = vk[LBM_VERT_RCPG * VS];
      float fu = v * absv + vb * vo - rcpg * (tv * pixb + tvdev * pix);
      float fv = -u * absv - ub * vo - rcpg * (tv * piyb + tvdev * piy);
      fu += vadv_p(rm[SF_U * I], u, rp[SF_U * I], sb0, sb1, hasm, hasp, dsk) +
            vadv_b(ub, hum, hup, sd0, sd1, hasm, hasp, dsk);
      fv += vadv_p(rm[SF_V * I], v, rp[SF_V * I], sb0, sb1, hasm, hasp, dsk) +
            vadv_b(vb, hvm, hvp, sd0, sd1, hasm, hasp, dsk);
      go[4 * I] = fu;
      go[5 * I] = fv;
      float ke = phiv + u * ub + v * vb;
      if (!d.strictly_linear) ke += 0.5f * (u * u + v * v);
      go[6 * I] = ke;
      go[7 * I] = v * tdev + vb * tt;
      go[2 * I] = q * divb + qb * dv +
                  vadv_p(rm[SF_Q * I], q, rp[SF_Q * I], sb0, sb1, hasm, hasp, dsk) +
                  vadv_b(qb, hqm, hqp, sd0, sd1, hasm, hasp, dsk);
      go[3 * I] = u * qb + ub * q;
      go[8 * I] = v * qb + vb * q;
    }
    __syncthreads();
    dft_fold<I>(fw, kb * NG, gout);
    __syncthreads();
    // quads: 2l -> (gt, xu, g, yu) of level l; 2l+1 -> (fu, fv, ke, xv); 2kb -> yv's
    dft_forward<I>(
        tab, fw, 2 * kb + 1, M,
        [&](int q, int k) -> int {
          if (q < 2 * kb) return (q >> 1) * NG + ((q & 1) ? 4 + k : k);
          return k < kb ? k * NG + 8 : -1;
        },
        [&](int q, int m, const int* fi, const float2* X) {
          const float rm = float(m);
          if (q < 2 * kb) {
            const int l = q >> 1;
            float2* o = fout + (size_t)(l * AF_N) * M;
            if ((q & 1) == 0) {
              // a3 = wg X(gt) - wd i m X(xu); a5 = wg X(g) - wd i m X(yu)
              o[AF_T * M + m] = make_float2(wg * X[0].x + wd * rm * X[1].y,
                                            wg * X[0].y - wd * rm * X[1].x);
              o[AF_Q * M + m] = make_float2(wg * X[2].x + wd * rm * X[3].y,
                                            wg * X[2].y - wd * rm * X[3].x);
            } else {
              o[AF_FU * M + m] = make_float2(wd * X[0].x, wd * X[0].y);
              o[AF_FV * M + m] = make_float2(wd * X[1].x, wd * X[1].y);
              o[AF_KE * M + m] = make_float2(wg * X[2].x, wg * X[2].y);
              o[AF_XV * M + m] = make_float2(wd * X[3].x, wd * X[3].y);
            }
          } else {
            for (int k = 0; k < kb; ++k)
              fout[(size_t)(k * AF_N + AF_YV) * M + m] = make_float2(wd * X[k].x, wd * X[k].y);
          }
        });
    __syncthreads();
    const int row = kb * AF_N;
    for (int m = warp; m < M; m += NW) {
      float2* dst = afe + ((size_t)m * J + j) * K * AF_N + (size_t)k0 * AF_N;
      for (int c = lane; c < row; c += 32) dst[c] = fout[c * M + m];
    }
  }
}

}  // namespace lbm
