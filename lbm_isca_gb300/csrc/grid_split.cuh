// FP32 grid-point step split into three kernels with full-size work per
// launch (included by stepper.cu):
//
//   k_idft  per (latitude, member): the longitude synthesis of the six
//           surface rows and the 6 K level rows of sf/sfs -> grid6
//           [E][J][6 + 6K][I] (surface pi, pi_x, pi_y, U-sum, V-sum, D-sum,
//           then per level u cos-scaled, v, vor, div, T, q);
//   k_alg   one thread per grid column: the grid-point algebra of
//           dynamics.py:176-262 in one upward pass over the levels (sigma-dot,
//           the reference-temperature split of the temperature equation and the
//           hydrostatic prefix running in registers) -> grid9
//           [E][J][2 + 9K][I] (gt_pi, pi(t-dt), then per level gt, xu, g, yu,
//           fu, fv, ke, xv, yv), plus the grid ps Robert-Asselin update;
//   k_fdft  per (latitude, member): the weighted longitude analysis of grid9
//           -> af/afs.
//
// The longitude transforms are dense DFTs folded by quarter-wave symmetry:
// the points i, I - i, I/2 - i, I/2 + i share |cos| and |sin| of every
// wavenumber, so even and odd m are accumulated apart over i <= I/4.

namespace lbm {

constexpr int SPLIT_NT = 256;
constexpr int IDFT_RC = 64;      // rows per staged chunk
constexpr int IDFT_RG = 8;       // rows per thread item

LBM_HD int idft_rows(int K) { return 6 + 6 * K; }
LBM_HD int fdft_rows(int K) { return 2 + 9 * K; }

LBM_HD size_t idft_smem(int I, int M) {
  const int Q = I / 4;
  const size_t tab = (size_t)M * (Q + 1) * sizeof(float2);
  return ((tab + 15) & ~size_t(15)) + 2 * (size_t)M * IDFT_RC * sizeof(float2);
}

// ---------------------------------------------------------------------------
template <int I>
__global__ void __launch_bounds__(SPLIT_NT) k_idft(SD<float> d, const float2* __restrict__ dft) {
  constexpr int Q = I / 4, NT = SPLIT_NT, RC = IDFT_RC, RG = IDFT_RG;
  const int j = blockIdx.x, e = blockIdx.y;
  const int J = d.J, K = d.K, M = d.M;
  const int NR = idft_rows(K);
  const int tid = threadIdx.x;
  extern __shared__ float4 sm4[];
  float2* tab = reinterpret_cast<float2*>(sm4);                       // [M][Q+1]
  float2* fin = reinterpret_cast<float2*>(
      reinterpret_cast<unsigned char*>(sm4) +
      (((size_t)M * (Q + 1) * sizeof(float2) + 15) & ~size_t(15)));  // [2][M][RC]
  for (int x = tid; x < M * (Q + 1); x += NT) tab[x] = dft[x];
  const float rcos = d.jfac[JF_RCOS * J + j];
  const float2* sfe = reinterpret_cast<const float2*>(d.sf) + (size_t)e * M * J * K * SF_N;
  const float2* sfs = reinterpret_cast<const float2*>(d.sfs);
  float* g6 = d.grid6 + ((size_t)e * J + j) * NR * I;

  // rows v0 .. v0 + RC - 1 of chunk into buffer b: level rows by cp.async (16
  // bytes = two rows of one m), the surface rows (chunk 0) by plain loads
  auto stage = [&](int v0, int b) {
    float2* F = fin + b * M * RC;
    const int vs = max(v0, 6), ve = min(v0 + RC, NR);
    if (ve > vs) {
      const int half = (ve - vs) >> 1;           // (ve - vs) and (vs - 6) are even
      for (int x = tid; x < M * half; x += NT) {
        const int m = x / half, c = 2 * (x - m * half);
        cp_async16(F + m * RC + (vs - v0) + c,
                   sfe + ((size_t)m * J + j) * K * SF_N + (vs - 6) + c);
      }
    }
    cp_async_commit();
    if (v0 == 0) {
      for (int x = tid; x < M * SFS_N; x += NT) {
        const int m = x / SFS_N, f = x - m * SFS_N;
        const float2 X = sfs[(((size_t)e * M + m) * J + j) * SFS_N + f];
        if (f == SFS_PI) {
          F[m * RC + 0] = X;
          F[m * RC + 1] = make_float2(-X.y * m * rcos, X.x * m * rcos);
        } else {
          const float s = (f == SFS_DH) ? 1.f : rcos;
          F[m * RC + f + 1] = make_float2(X.x * s, X.y * s);
        }
      }
    }
  };
  // longitude scale of row v: u cos and v cos rows take 1 / (a cos)
  auto rscale = [&](int v) -> float {
    if (v < 6) return 1.f;
    const int f = (v - 6) % SF_N;
    return (f == SF_U || f == SF_V) ? rcos : 1.f;
  };

  stage(0, 0);
  int buf = 0;
  for (int v0 = 0; v0 < NR; v0 += RC) {
    const int nr = min(RC, NR - v0);
    if (v0 + RC < NR) stage(v0 + RC, buf ^ 1);
    else cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const float2* F = fin + buf * M * RC;
    // points i = 1..Q, RG rows per item: x_i, x_{I-i}, x_{I/2-i}, x_{I/2+i}
    constexpr int NGR = RC / RG;
    for (int it = tid; it < Q * NGR; it += NT) {
      const int i = it % Q + 1, g = it / Q;
      const int r0 = g * RG;
      if (r0 >= nr) continue;
      float ce[RG], co[RG], se[RG], so[RG];
#pragma unroll
      for (int r = 0; r < RG; ++r) ce[r] = co[r] = se[r] = so[r] = 0.f;
      const float2* tb = tab + i;
      int m = 1;
      for (; m + 1 < M; m += 2) {              // (odd, even) pairs of m >= 1
        const float2 to = tb[m * (Q + 1)], te = tb[(m + 1) * (Q + 1)];
        const float4* xo = reinterpret_cast<const float4*>(F + m * RC + r0);
        const float4* xe = reinterpret_cast<const float4*>(F + (m + 1) * RC + r0);
#pragma unroll
        for (int t = 0; t < RG / 2; ++t) {
          const float4 b = xo[t], a = xe[t];
          co[2 * t] = fmaf(b.x, to.x, co[2 * t]);       so[2 * t] = fmaf(b.y, to.y, so[2 * t]);
          co[2 * t + 1] = fmaf(b.z, to.x, co[2 * t + 1]); so[2 * t + 1] = fmaf(b.w, to.y, so[2 * t + 1]);
          ce[2 * t] = fmaf(a.x, te.x, ce[2 * t]);       se[2 * t] = fmaf(a.y, te.y, se[2 * t]);
          ce[2 * t + 1] = fmaf(a.z, te.x, ce[2 * t + 1]); se[2 * t + 1] = fmaf(a.w, te.y, se[2 * t + 1]);
        }
      }
      if (m < M) {                              // last (odd) m
        const float2 to = tb[m * (Q + 1)];
        const float4* xo = reinterpret_cast<const float4*>(F + m * RC + r0);
#pragma unroll
        for (int t = 0; t < RG / 2; ++t) {
          const float4 b = xo[t];
          co[2 * t] = fmaf(b.x, to.x, co[2 * t]);       so[2 * t] = fmaf(b.y, to.y, so[2 * t]);
          co[2 * t + 1] = fmaf(b.z, to.x, co[2 * t + 1]); so[2 * t + 1] = fmaf(b.w, to.y, so[2 * t + 1]);
        }
      }
#pragma unroll
      for (int r = 0; r < RG; ++r) {
        if (r0 + r >= nr) break;
        const int v = v0 + r0 + r;
        const float sc = rscale(v);
        const float c0 = F[r0 + r].x + 2.f * ce[r], c1 = 2.f * co[r];
        const float s0 = 2.f * se[r], s1 = 2.f * so[r];
        const float p = c0 + c1, mn = c0 - c1, s = s0 + s1, dd = s0 - s1;
        float* row = g6 + (size_t)v * I;
        row[i] = (p - s) * sc;
        row[I - i] = (p + s) * sc;
        row[I / 2 - i] = (mn + dd) * sc;
        row[I / 2 + i] = (mn - dd) * sc;
      }
    }
    // i = 0 and i = I/2: one row per thread (consecutive rows, no bank conflicts)
    for (int r = tid; r < nr; r += NT) {
      float se_ = 0.f, so_ = 0.f;
      for (int m = 1; m < M; ++m) {
        const float a = F[m * RC + r].x;
        if (m & 1) so_ += a;
        else se_ += a;
      }
      const int v = v0 + r;
      const float sc = rscale(v), x0 = F[r].x;
      g6[(size_t)v * I] = (x0 + 2.f * (se_ + so_)) * sc;
      g6[(size_t)v * I + I / 2] = (x0 + 2.f * (se_ - so_)) * sc;
    }
    buf ^= 1;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// One thread per column (blockDim = I).
template <int I>
__global__ void __launch_bounds__(I) k_alg(SD<float> d, int ps_mode) {
  const int j = blockIdx.x, e = blockIdx.y, c = threadIdx.x;
  const int J = d.J, K = d.K;
  __shared__ float vert[LBM_VERT_COUNT * 65];
  for (int x = c; x < LBM_VERT_COUNT * (K + 1); x += I) vert[x] = d.vert[x];
  __syncthreads();
  const int VS = K + 1;
  auto V = [&](int row, int k) { return vert[row * VS + k]; };
  const float* g6 = d.grid6 + ((size_t)e * J + j) * idft_rows(K) * I + c;
  float* g9 = d.grid9 + ((size_t)e * J + j) * fdft_rows(K) * I + c;
  const float eps = d.epsvt, kappa = d.kappa;

  // ---- surface: column sums, pi tendency, grid ps filter ----
  const size_t g2 = (size_t)j * I + c;
  const float* b2 = d.b2;
  const float pixb = b2[(B2_PIX * J) * I + g2], piyb = b2[(B2_PIY * J) * I + g2];
  const float psbar = b2[(B2_PSBAR * J) * I + g2];
  const float usum = b2[(B2_USUM * J) * I + g2], vsum = b2[(B2_VSUM * J) * I + g2];
  const float pi = g6[0], pix = g6[I], piy = g6[2 * I];
  const float uh = g6[3 * I], vh = g6[4 * I], dh = g6[5 * I];
  const float sx = pixb * uh + piyb * vh + pix * usum + piy * vsum;   // sum dsig v.grad(pi)
  const float stot = dh + sx;
  g9[0] = -sx;                                   // gt_pi
  {
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
    g9[I] = log1pf(pb / psbar);                  // pi(t - dt)
  }

  // ---- levels, bottom up ----
  // per-field offsets into b3 (int: the basic state of one latitude is small)
  const int b3f = J * K * I;
  const float* bk = d.b3 + (size_t)j * K * I + c;             // level k, field 0
  const float* bsk = d.bsd + (size_t)j * (K + 1) * I + c;     // interface k
  const float* gl = g6 + (size_t)6 * I;                       // level k rows
  float* go = g9 + (size_t)2 * I;
  float sdlo = (V(LBM_VERT_SIGM, 0) - 1.f) * stot;   // sigma-dot at k - 1/2
  float prefd = 0.f, prefp = 0.f, pref3 = 0.f;
  // level window: m = k-1, 0 = k, p = k+1 (u, v, T, q); vorticity and
  // divergence of level k only
  float um = 0.f, vm = 0.f, tm_ = 0.f, qm = 0.f;
  float u0 = gl[SF_U * I], v0 = gl[SF_V * I], t0 = gl[SF_T * I], q0 = gl[SF_Q * I];
  float vo0 = gl[SF_VOR * I], dv0 = gl[SF_DIV * I];
  float hum = 0.f, hvm = 0.f, htm = 0.f, hqm = 0.f;    // half differences at k - 1
  float sb0 = __ldg(bsk);
  for (int k = 0; k < K; ++k) {
    const bool hasm = k >= 1, hasp = k + 1 <= K - 1;
    float up = u0, vp = v0, tp = t0, qp = q0, vop = 0.f, dvp = 0.f;
    if (hasp) {
      const float* gn = gl + SF_N * I;
      up = gn[SF_U * I]; vp = gn[SF_V * I]; tp = gn[SF_T * I]; qp = gn[SF_Q * I];
      vop = gn[SF_VOR * I]; dvp = gn[SF_DIV * I];
    }
    const float ub = __ldg(bk + B_U * b3f), vb = __ldg(bk + B_V * b3f);
    const float tb = __ldg(bk + B_T * b3f), qb = __ldg(bk + B_Q * b3f);
    const float tvb = __ldg(bk + B_TV * b3f), absv = __ldg(bk + B_ABSVOR * b3f);
    const float divb = __ldg(bk + B_DIV * b3f), x5b = __ldg(bk + B_X5 * b3f);
    const float tdev = __ldg(bk + B_TDEV * b3f), tvdev = __ldg(bk + B_TVDEV * b3f);
    const float hup = __ldg(bk + B_HDU * b3f), hvp = __ldg(bk + B_HDV * b3f);
    const float htp = __ldg(bk + B_HDT * b3f), hqp = __ldg(bk + B_HDQ * b3f);
    const float sb1 = __ldg(bsk + I);
    const float dsk = V(LBM_VERT_DSIG, k), rdsk = 1.f / dsk;
    // column scans through level k
    const float pa = u0 * pixb + ub * pix + v0 * piyb + vb * piy;      // v.grad(pi)
    const float sdup = sdlo + dsk * (dv0 + pa - stot);               // sigma-dot at k + 1/2
    prefd += dsk * dv0;
    prefp += dsk * pa;
    const float xv = eps * (t0 * qb + tb * q0);                       // Tv' - T'
    const float phiv = pref3 + V(LBM_VERT_RALPHA, k) * xv;             // (WW (Tv'-T'))_k
    pref3 += V(LBM_VERT_RDLOG3, k) * xv;
    const float sdv = dh - prefd, spv = sx - prefp;                   // suffix sums above k
    const float sd0 = hasm ? sdlo : 0.f, sd1 = hasp ? sdup : 0.f;
    // vertical advection of dynamics.py's _vert_advect written in differences,
    //   (s1 (f[k+1] - f[k]) / 2 + s0 (f[k] - f[k-1]) / 2) / dsig_k
    // (at the bottom / top the missing half becomes +s0 f[k] / -s1 f[k]),
    // equal to the flux form (F[k+1/2] - F[k-1/2] - f[k] (s1 - s0)) / dsig_k
    // without cancelling the f[k] (s1 - s0) part: perturbation fields by the
    // basic sigma-dot, basic fields (half differences precomputed in FP64)
    // by sigma-dot'
    auto vp_ = [&](float fm, float f0, float fp) {
      const float a = hasp ? 0.5f * sb1 * (fp - f0) : -sb1 * f0;
      const float b = hasm ? 0.5f * sb0 * (f0 - fm) : sb0 * f0;
      return (a + b) * rdsk;
    };
    auto vb_ = [&](float f0, float hm, float hp) {
      const float a = hasp ? sd1 * hp : -sd1 * f0;
      const float b = hasm ? sd0 * hm : sd0 * f0;
      return (a + b) * rdsk;
    };
    // temperature: adiabatic term and the reference-temperature matrix with
    // Tref cancelled algebraically
    const float tv = t0 + xv;
    const float al = V(LBM_VERT_ALPHA, k), w3 = V(LBM_VERT_W3, k);
    const float adtm = -kappa * (tv * x5b + tvdev * (al * dv0 + w3 * sdv) +
                                 tvb * (V(LBM_VERT_WP, k) * pa + w3 * spv));
    const float hadv = t0 * divb + tdev * dv0;
    go[0 * I] = adtm + hadv + vp_(tm_, t0, tp) + vb_(tb, htm, htp);  // gt
    go[1 * I] = u0 * tdev + ub * t0;                                  // xu
    const float rcpg = V(LBM_VERT_RCPG, k);
    const float fu = v0 * absv + vb * vo0 - rcpg * (tv * pixb + tvdev * pix) +
                     vp_(um, u0, up) + vb_(ub, hum, hup);
    const float fv = -u0 * absv - ub * vo0 - rcpg * (tv * piyb + tvdev * piy) +
                     vp_(vm, v0, vp) + vb_(vb, hvm, hvp);
    go[4 * I] = fu;
    go[5 * I] = fv;
    float ke = phiv + u0 * ub + v0 * vb;
    if (!d.strictly_linear) ke += 0.5f * (u0 * u0 + v0 * v0);
    go[6 * I] = ke;
    go[7 * I] = v0 * tdev + vb * t0;                                  // xv
    go[2 * I] = q0 * divb + qb * dv0 + vp_(qm, q0, qp) + vb_(qb, hqm, hqp);   // g
    go[3 * I] = u0 * qb + ub * q0;                                    // yu
    go[8 * I] = v0 * qb + vb * q0;                                    // yv
    // advance the window
    um = u0; vm = v0; tm_ = t0; qm = q0;
    u0 = up; v0 = vp; t0 = tp; q0 = qp; vo0 = vop; dv0 = dvp;
    hum = hup; hvm = hvp; htm = htp; hqm = hqp;
    sdlo = sdup;
    sb0 = sb1;
    bk += I;
    bsk += I;
    gl += SF_N * I;
    go += 9 * I;
  }
}

// ---------------------------------------------------------------------------
// Longitude analysis.  A chunk of LC levels at a time: the 9 LC grid rows
// (and in the first chunk the two surface rows) stream into shared memory by
// cp.async while the previous chunk computes, are folded by quarter-wave
// symmetry into fw[row][i] = (u+uh, u-uh, v-vh, v+vh) (u, v: sum / difference
// of x_i and x_{I-i}; uh, vh: of x_{I/2-i} and x_{I/2+i}), and each thread
// item accumulates one "quad" of 4 rows against one wavenumber pair (m even,
// m odd), reading one packed table entry (cos, sin of the even m, cos, sin of
// the odd m) per point.
LBM_HD int fdft_quads(int lc) { return 2 * lc + (lc + 3) / 4; }

struct FdftLayout {
  int tab, raw, fw, fout, total;     // float units, 16-byte aligned blocks
  LBM_HD static int al4(int x) { return (x + 3) & ~3; }
  LBM_HD FdftLayout(int I, int M, int LC) {
    const int Q = I / 4, NP = (M + 1) / 2, NR = 9 * LC + 2;
    int o = 0;
    tab = o; o = al4(o + 4 * NP * (Q + 1));
    raw = o; o = al4(o + NR * I);
    fw = o; o = al4(o + 4 * NR * (Q + 1));
    fout = o; o = al4(o + 2 * LC * AF_N * M);
    total = o;
  }
};

// Level chunk: as many levels as keep the thread items of a chunk within one
// pass of the block and the shared memory within 74 KB (three CTAs on an SM),
// then evened out over the chunks.
LBM_HD int fdft_chunk(int I, int M, int K) {
  const int NP = (M + 1) / 2;
  int lc = K;
  while (lc > 1 && ((fdft_quads(lc) + 1) * NP > SPLIT_NT ||
                    sizeof(float) * (size_t)FdftLayout(I, M, lc).total > 74 * 1024))
    --lc;
  const int nchunk = (K + lc - 1) / lc;
  return (K + nchunk - 1) / nchunk;
}

template <int I>
__global__ void __launch_bounds__(SPLIT_NT) k_fdft(SD<float> d, const float2* __restrict__ dft,
                                                  int LC) {
  constexpr int Q = I / 4, NT = SPLIT_NT, NW = NT / 32;
  const int j = blockIdx.x, e = blockIdx.y;
  const int J = d.J, K = d.K, M = d.M, NP = (M + 1) / 2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const FdftLayout L(I, M, LC);
  extern __shared__ float4 sm4[];
  float* sm = reinterpret_cast<float*>(sm4);
  float4* tab = reinterpret_cast<float4*>(sm + L.tab);     // [NP][Q+1]
  float* raw = sm + L.raw;                                 // [rows][I]
  float4* fw = reinterpret_cast<float4*>(sm + L.fw);       // [rows][Q+1]
  float2* fout = reinterpret_cast<float2*>(sm + L.fout);   // [LC*7][M]
  for (int x = tid; x < NP * (Q + 1); x += NT) {
    const int p = x / (Q + 1), i = x - p * (Q + 1);
    const float2 te = dft[(2 * p) * (Q + 1) + i];
    const float2 to = (2 * p + 1 < M) ? dft[(2 * p + 1) * (Q + 1) + i] : make_float2(0.f, 0.f);
    tab[x] = make_float4(te.x, te.y, to.x, to.y);
  }
  const float gw = d.jfac[JF_GW * J + j], gwdc = d.jfac[JF_GWDELC * J + j];
  const float wg = gw / float(I), wd = gwdc / float(I);
  const float* g9 = d.grid9 + ((size_t)e * J + j) * fdft_rows(K) * I;
  float2* afe = reinterpret_cast<float2*>(d.af) + (size_t)e * M * J * K * AF_N;
  // rows of the chunk at k0: level rows 0 .. 9 lc - 1, then (first chunk)
  // the two surface rows
  auto stage = [&](int k0) {
    const int lc = min(LC, K - k0);
    const float* src = g9 + (size_t)(2 + 9 * k0) * I;
    const int n4 = 9 * lc * I / 4;
    for (int x = tid; x < n4; x += NT) cp_async16(raw + 4 * x, src + 4 * x);
    if (k0 == 0)
      for (int x = tid; x < 2 * I / 4; x += NT) cp_async16(raw + 9 * lc * I + 4 * x, g9 + 4 * x);
    cp_async_commit();
  };
  stage(0);
  for (int k0 = 0; k0 < K; k0 += LC) {
    const int lc = min(LC, K - k0);
    const bool surf = (k0 == 0);
    const int nrow = 9 * lc + (surf ? 2 : 0);
    cp_async_wait<0>();
    __syncthreads();
    for (int x = tid; x < nrow * (Q + 1); x += NT) {
      const int r = x / (Q + 1), i = x - r * (Q + 1);
      const float* row = raw + r * I;
      float4 v;
      if (i == 0) {
        const float xq = row[Q], x3q = row[3 * Q];
        v = make_float4(row[0], row[I / 2], xq + x3q, xq - x3q);
      } else if (i == Q) {
        v = make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
        const float xa = row[i], xb = row[I - i], xc = row[I / 2 - i], xd = row[I / 2 + i];
        const float u = xa + xb, w = xa - xb, uh = xc + xd, vh = xc - xd;
        v = make_float4(u + uh, u - uh, w - vh, w + vh);
      }
      fw[x] = v;
    }
    __syncthreads();
    if (k0 + LC < K) stage(k0 + LC);             // next chunk streams in meanwhile
    const int nq = fdft_quads(lc) + (surf ? 1 : 0);
    for (int it = tid; it < nq * NP; it += NT) {
      const int p = it % NP, q = it / NP;
      // rows of quad q (-1: none)
      int rw[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        if (q < 2 * lc) {
          rw[t] = 9 * (q >> 1) + ((q & 1) ? 4 : 0) + t;
        } else if (q < fdft_quads(lc)) {
          const int l = 4 * (q - 2 * lc) + t;
          rw[t] = l < lc ? 9 * l + 8 : -1;
        } else {
          rw[t] = t < 2 ? 9 * lc + t : -1;
        }
      }
      const float4* w[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) w[t] = fw + (rw[t] >= 0 ? rw[t] : 0) * (Q + 1);
      float acc[4][4];
#pragma unroll
      for (int t = 0; t < 4; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
      const float4* tb = tab + p * (Q + 1);
#pragma unroll 4
      for (int i = 1; i < Q; ++i) {
        const float4 c = tb[i];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const float4 a = w[t][i];
          acc[t][0] = fmaf(a.x, c.x, acc[t][0]);   // even m: cos
          acc[t][1] = fmaf(a.z, c.y, acc[t][1]);   // even m: sin
          acc[t][2] = fmaf(a.y, c.z, acc[t][2]);   // odd m: cos
          acc[t][3] = fmaf(a.w, c.w, acc[t][3]);   // odd m: sin
        }
      }
      const int me = 2 * p, mo = 2 * p + 1;
      const float ce = (p & 1) ? -1.f : 1.f;            // (-1)^{me/2}
      const float so = (((mo - 1) / 2) & 1) ? -1.f : 1.f;  // (-1)^{(mo-1)/2}
      float2 Xe[4], Xo[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const float4 b0 = w[t][0];        // (x0, x_{I/2}, u_Q, v_Q)
        Xe[t] = make_float2(acc[t][0] + b0.x + b0.y + ce * b0.z, -acc[t][1]);
        Xo[t] = make_float2(acc[t][2] + b0.x - b0.y, -(acc[t][3] + so * b0.w));
      }
      // I X_m of the quad's rows -> weighted analysis inputs
      for (int par = 0; par < 2; ++par) {
        const int m = par ? mo : me;
        if (m >= M) break;
        const float2* X = par ? Xo : Xe;
        const float rm = float(m);
        if (q < 2 * lc) {
          float2* o = fout + ((q >> 1) * AF_N) * M;
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
        } else if (q < fdft_quads(lc)) {
          for (int t = 0; t < 4; ++t) {
            const int l = 4 * (q - 2 * lc) + t;
            if (l < lc) fout[(l * AF_N + AF_YV) * M + m] = make_float2(wd * X[t].x, wd * X[t].y);
          }
        } else {
          float2* o = reinterpret_cast<float2*>(d.afs) + (((size_t)e * M + m) * J + j) * 2;
          o[0] = make_float2(X[0].x * wg, X[0].y * wg);
          o[1] = make_float2(X[1].x * wg, X[1].y * wg);
        }
      }
    }
    __syncthreads();
    const int row = lc * AF_N;
    for (int m = warp; m < M; m += NW) {
      float2* dst = afe + ((size_t)m * J + j) * K * AF_N + (size_t)k0 * AF_N;
      for (int c = lane; c < row; c += 32) dst[c] = fout[c * M + m];
    }
  }
}

}  // namespace lbm
