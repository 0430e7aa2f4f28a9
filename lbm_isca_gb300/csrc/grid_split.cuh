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
//   k_fdft  persistent CTAs over (member, latitude, level chunk) units: the
//           weighted longitude analysis of grid9 -> af/afs as four
//           register-tiled plane products (see the kernel).
//
// The longitude transforms are dense DFTs folded by quarter-wave symmetry:
// the points i, I - i, I/2 - i, I/2 + i share |cos| and |sin| of every
// wavenumber, so even and odd m are accumulated apart over i <= I/4.

namespace lbm {

constexpr int IDFT_NT = 128;    // threads of the longitude synthesis block
constexpr int IDFT_RC = 48;      // rows per staged chunk (two buffers fit five CTAs per SM)
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
__global__ void __launch_bounds__(IDFT_NT) k_idft(SD<float> d, const float2* __restrict__ dft) {
  constexpr int Q = I / 4, NT = IDFT_NT, RC = IDFT_RC, RG = IDFT_RG;
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
    // points i and i + Q/2 (1 <= i <= Q/2), RG rows per item: each point
    // gives x_i, x_{I-i}, x_{I/2-i}, x_{I/2+i}; a row value read from shared
    // memory serves both points
    constexpr int NGR = RC / RG, QH = Q / 2;
    for (int it = tid; it < QH * NGR; it += NT) {
      const int i0 = it % QH + 1, g = it / QH;
      const int r0 = g * RG;
      if (r0 >= nr) continue;
      float ce[2][RG], co[2][RG], se[2][RG], so[2][RG];
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int r = 0; r < RG; ++r) ce[h][r] = co[h][r] = se[h][r] = so[h][r] = 0.f;
      const float2* tb0 = tab + i0;
      const float2* tb1 = tab + i0 + QH;
      int m = 1;
      for (; m + 1 < M; m += 2) {              // (odd, even) pairs of m >= 1
        const float2 to0 = tb0[m * (Q + 1)], te0 = tb0[(m + 1) * (Q + 1)];
        const float2 to1 = tb1[m * (Q + 1)], te1 = tb1[(m + 1) * (Q + 1)];
        const float4* xo = reinterpret_cast<const float4*>(F + m * RC + r0);
        const float4* xe = reinterpret_cast<const float4*>(F + (m + 1) * RC + r0);
#pragma unroll
        for (int t = 0; t < RG / 2; ++t) {
          const float4 b = xo[t], a = xe[t];
          co[0][2 * t] = fmaf(b.x, to0.x, co[0][2 * t]);       so[0][2 * t] = fmaf(b.y, to0.y, so[0][2 * t]);
          co[0][2 * t + 1] = fmaf(b.z, to0.x, co[0][2 * t + 1]); so[0][2 * t + 1] = fmaf(b.w, to0.y, so[0][2 * t + 1]);
          ce[0][2 * t] = fmaf(a.x, te0.x, ce[0][2 * t]);       se[0][2 * t] = fmaf(a.y, te0.y, se[0][2 * t]);
          ce[0][2 * t + 1] = fmaf(a.z, te0.x, ce[0][2 * t + 1]); se[0][2 * t + 1] = fmaf(a.w, te0.y, se[0][2 * t + 1]);
          co[1][2 * t] = fmaf(b.x, to1.x, co[1][2 * t]);       so[1][2 * t] = fmaf(b.y, to1.y, so[1][2 * t]);
          co[1][2 * t + 1] = fmaf(b.z, to1.x, co[1][2 * t + 1]); so[1][2 * t + 1] = fmaf(b.w, to1.y, so[1][2 * t + 1]);
          ce[1][2 * t] = fmaf(a.x, te1.x, ce[1][2 * t]);       se[1][2 * t] = fmaf(a.y, te1.y, se[1][2 * t]);
          ce[1][2 * t + 1] = fmaf(a.z, te1.x, ce[1][2 * t + 1]); se[1][2 * t + 1] = fmaf(a.w, te1.y, se[1][2 * t + 1]);
        }
      }
      if (m < M) {                              // last (odd) m
        const float2 to0 = tb0[m * (Q + 1)], to1 = tb1[m * (Q + 1)];
        const float4* xo = reinterpret_cast<const float4*>(F + m * RC + r0);
#pragma unroll
        for (int t = 0; t < RG / 2; ++t) {
          const float4 b = xo[t];
          co[0][2 * t] = fmaf(b.x, to0.x, co[0][2 * t]);       so[0][2 * t] = fmaf(b.y, to0.y, so[0][2 * t]);
          co[0][2 * t + 1] = fmaf(b.z, to0.x, co[0][2 * t + 1]); so[0][2 * t + 1] = fmaf(b.w, to0.y, so[0][2 * t + 1]);
          co[1][2 * t] = fmaf(b.x, to1.x, co[1][2 * t]);       so[1][2 * t] = fmaf(b.y, to1.y, so[1][2 * t]);
          co[1][2 * t + 1] = fmaf(b.z, to1.x, co[1][2 * t + 1]); so[1][2 * t + 1] = fmaf(b.w, to1.y, so[1][2 * t + 1]);
        }
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = i0 + h * QH;
#pragma unroll
        for (int r = 0; r < RG; ++r) {
          if (r0 + r >= nr) break;
          const int v = v0 + r0 + r;
          const float sc = rscale(v);
          const float c0 = F[r0 + r].x + 2.f * ce[h][r], c1 = 2.f * co[h][r];
          const float s0 = 2.f * se[h][r], s1 = 2.f * so[h][r];
          const float p = c0 + c1, mn = c0 - c1, s = s0 + s1, dd = s0 - s1;
          float* row = g6 + (size_t)v * I;
          row[i] = (p - s) * sc;
          row[I - i] = (p + s) * sc;
          row[I / 2 - i] = (mn + dd) * sc;
          row[I / 2 + i] = (mn - dd) * sc;
        }
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
// One thread per column (blockDim = I).  The kernel waits on global loads;
// the minimum resident blocks per SM keep 92 / 80 / 80 registers at I = 64 /
// 128 / 256 -- at 128 that is six blocks instead of five, 10% faster at 512
// members (seven and eight spill and are slower).
template <int I>
__global__ void __launch_bounds__(I, I == 64 ? 10 : (I == 128 ? 6 : 3))
    k_alg(SD<float> d, int ps_mode) {
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
// Longitude analysis, written as four register-tiled products of folded grid
// rows with the folded DFT table.
//
// Work unit: the rows of LC levels of one (member, latitude) column (the 9 LC
// level rows gt xu g yu fu fv ke xv yv per level, and in the unit of level 0
// the two surface rows).  Each row is folded by quarter-wave symmetry into
// four planes over the points 0 < i < I/4, with u, w the sum / difference of
// x_i and x_{I-i} and uh, vh those of x_{I/2-i} and x_{I/2+i}:
//   P0 = u + uh (cos, even m)  P1 = w - vh (sin, even m)
//   P2 = u - uh (cos, odd m)   P3 = w + vh (sin, odd m)
// and the table likewise into T0..T3 = cos, sin of m = 2p and of m = 2p + 1.
// Plane c gives the sums S_c[row][p] = sum_i P_c[i][row] T_c[i][p]; each lane
// owns one c and an 8-row by 8-pair tile (64 accumulators) and reads per point
// two float4 of its rows and two of its pairs.  The quarter warps of a half
// warp hold different planes, so every 16-byte load is one shared-memory
// wavefront per half warp (conflict-free by the plane and row strides).  The
// sums go through shared memory to an output pass that combines rows (a3 =
// wg X(gt) - wd i m X(xu), ...) and writes af/afs with coalesced stores.
//
// CTAs are persistent: each walks the units with a grid stride, loads the
// table once, and streams the next unit's rows into shared memory by
// cp.async while it computes the current one.
struct FdftPlan {
  int lc, nrg, npg, warps, nt;           // levels, row groups, pair groups, warps, threads
  int rp, ps, npp, ts;                   // strides (floats): plane point, plane, table point,
                                         //   table plane
  int tab, pl, b0, total;                // float offsets of the shared-memory blocks, size
};

LBM_HD FdftPlan fdft_layout(int I, int M, int lc) {
  const int Q = I / 4, NP = (M + 1) / 2, nrow = 9 * lc + 2;
  FdftPlan p;
  p.lc = lc;
  p.nrg = (nrow + 7) / 8;
  p.npg = (NP + 7) / 8;
  p.warps = (p.nrg * p.npg + 7) / 8;
  p.nt = 32 * p.warps;
  p.rp = 8 * p.nrg + 4;                             // = 4 (mod 8): conflict-free fold stores
  p.ps = Q * p.rp + 4;                              // = 4 (mod 8): planes c, c+1 apart
  p.npp = 8 * p.npg;
  p.ts = Q * p.npp + 4;
  auto al4 = [](int x) { return (x + 3) & ~3; };
  // the staged outputs [M][7 lc] float2 alias the planes
  int planes = 4 * p.ps;
  if (14 * M * lc > planes) planes = 14 * M * lc;
  int o = 0;
  p.tab = o; o = al4(o + 4 * p.ts);
  p.pl = o; o = al4(o + planes);
  p.b0 = o; o = al4(o + 4 * 8 * p.nrg);
  p.total = o;
  return p;
}

// Levels per unit, evened out over the units of a column: the best product of
// the useful fraction of the computed rows, the busy fraction of the lanes
// and the resident warps per SM (shared memory, 128 registers a thread; counted
// up to 12), more levels on a tie.
LBM_HD FdftPlan fdft_plan(int I, int M, int K) {
  float best_score = -1.f;
  int best = 0;
  for (int cand = 1; cand <= K; ++cand) {
    const int nch = (K + cand - 1) / cand, lc = (K + nch - 1) / nch;
    const FdftPlan p = fdft_layout(I, M, lc);
    const size_t sm = sizeof(float) * (size_t)p.total;
    if (p.warps > 8 || sm > 227 * 1024) continue;
    int ctas = (int)((228 * 1024) / (sm + 1024));
    const int creg = 65536 / (p.nt * 128);
    if (creg < ctas) ctas = creg;
    if (32 / p.warps < ctas) ctas = 32 / p.warps;
    int w = ctas * p.warps;
    if (w > 12) w = 12;
    const float rows = float(9 * lc) / float(8 * p.nrg);
    const float lanes = float(p.nrg * p.npg) / float(8 * p.warps);
    const float score = rows * lanes * float(w);
    if (score >= best_score) { best_score = score; best = lc; }
  }
  if (best == 0) {
    FdftPlan none = fdft_layout(I, M, 1);
    none.total = 1 << 30;                  // nothing fits: rejected by the caller
    return none;
  }
  return fdft_layout(I, M, best);
}

template <int I>
__global__ void __launch_bounds__(256) k_fdft(SD<float> d, const float2* __restrict__ dft,
                                              FdftPlan pl) {
  constexpr int Q = I / 4;
  const int J = d.J, K = d.K, M = d.M, NR9 = fdft_rows(K);
  const int LC = pl.lc, RP = pl.rp, PS = pl.ps, NPP = pl.npp, TS = pl.ts;
  const int nt = blockDim.x, nwarp = pl.warps;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nch = (K + LC - 1) / LC, nunits = d.E * J * nch;
  extern __shared__ float4 sm4[];
  float* sm = reinterpret_cast<float*>(sm4);
  float* tab = sm + pl.tab;                 // [4][Q][NPP] (plane stride TS)
  float* pln = sm + pl.pl;                  // [4][Q][RP] (plane stride PS); later the sums
  float4* b0s = reinterpret_cast<float4*>(sm + pl.b0);   // [rows] (x0, x_{I/2}, u_Q, v_Q)

  for (int x = tid; x < Q * NPP; x += nt) {
    const int i = x / NPP, p = x - i * NPP;
    const int me = 2 * p, mo = 2 * p + 1;
    const float2 te = me < M ? dft[me * (Q + 1) + i] : make_float2(0.f, 0.f);
    const float2 to = mo < M ? dft[mo * (Q + 1) + i] : make_float2(0.f, 0.f);
    tab[0 * TS + x] = te.x;
    tab[1 * TS + x] = te.y;
    tab[2 * TS + x] = to.x;
    tab[3 * TS + x] = to.y;
  }

  // unit u: level chunk u % nch of column u / nch (member-major, then latitude)
  for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
    const int cu = u % nch, col = u / nch;
    const int e = col / J, j = col - e * J;
    const int k0 = cu * LC, lc = min(LC, K - k0);
    const bool surf = (cu == 0);
    const int nrow = 9 * lc + (surf ? 2 : 0);
    // unit rows: the level rows, then (level 0) the two surface rows
    const float* g9 = d.grid9 + (size_t)col * NR9 * I;
    const float* lev = g9 + (size_t)(2 + 9 * k0) * I;
    __syncthreads();                         // the previous unit's sums are read
    // fold: a lane takes one point of four consecutive plane rows (a warp:
    // 32 points, or two row quads at I = 64) and stores each plane's four
    // rows as one float4; the lanes of point 0 keep (x0, x_{I/2}, u_Q, v_Q).
    // Plane rows: level l's gt xu g yu fu fv ke xv at 8 l .. 8 l + 7, then the
    // yv rows of the levels, then (level 0) the two surface rows.
    {
      constexpr int PPW = Q < 32 ? Q : 32, SUB = 32 / PPW, NIW = Q / PPW;
      const int nrq = (nrow + 3) >> 2;
      const int nit = ((nrq + SUB - 1) / SUB) * NIW;
      auto rowp = [&](int pr) -> const float* {
        if (pr < 8 * lc) return lev + (size_t)(9 * (pr >> 3) + (pr & 7)) * I;
        if (pr < 9 * lc) return lev + (size_t)(9 * (pr - 8 * lc) + 8) * I;
        return g9 + (size_t)(pr - 9 * lc) * I;
      };
      for (int it = warp; it < nit; it += nwarp) {
        const int rq = (it / NIW) * SUB + lane / PPW;
        const int i = (it % NIW) * PPW + (lane & (PPW - 1));
        if (rq < nrq) {
          float xv[4][4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const int r = 4 * rq + t;
            if (r < nrow) {
              const float* row = rowp(r);
              xv[t][0] = __ldg(row + i);
              xv[t][1] = __ldg(row + ((I - i) & (I - 1)));
              xv[t][2] = __ldg(row + (I / 2 - i));
              xv[t][3] = __ldg(row + (I / 2 + i));
            } else {
              xv[t][0] = xv[t][1] = xv[t][2] = xv[t][3] = 0.f;
            }
          }
          float pv[4][4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const float xa = xv[t][0], xb = xv[t][1], xc = xv[t][2], xd = xv[t][3];
            const float uu = xa + xb, w = xa - xb, uh = xc + xd, vh = xc - xd;
            pv[0][t] = uu + uh;
            pv[1][t] = w - vh;
            pv[2][t] = uu - uh;
            pv[3][t] = w + vh;
            const int r = 4 * rq + t;
            if (i == 0 && r < nrow) {
              const float* row = rowp(r);
              const float xq = __ldg(row + Q), x3q = __ldg(row + 3 * Q);
              b0s[r] = make_float4(xa, xc, xq + x3q, xq - x3q);
            }
          }
          if (i != 0) {
            float* o = pln + i * RP + 4 * rq;
#pragma unroll
            for (int c = 0; c < 4; ++c)
              *reinterpret_cast<float4*>(o + c * PS) = make_float4(pv[c][0], pv[c][1], pv[c][2], pv[c][3]);
          }
        }
      }
    }
    __syncthreads();
    if (tid == 0 && u + (int)gridDim.x < nunits) {
      // the next unit's rows (contiguous level rows, surface rows) into L2
      const int un = u + gridDim.x, cn = un % nch, coln = un / nch;
      const int kn = cn * LC, lcn = min(LC, K - kn);
      const float* gn = d.grid9 + (size_t)coln * NR9 * I;
      prefetch_l2_bulk(gn + (size_t)(2 + 9 * kn) * I, 9u * lcn * I * sizeof(float));
      if (cn == 0) prefetch_l2_bulk(gn, 2u * I * sizeof(float));
    }

    // plane sums: lane = plane c (quarter warp) x (row group, pair group)
    const int c = lane >> 3, k = warp * 8 + (lane & 7);
    const int npg = pl.npg;
    const bool active = k < pl.nrg * npg;
    const int rg = active ? k / npg : 0, pg = active ? k - rg * npg : 0;
    // the sums start from the point-0 and point-I/4 terms of their plane:
    // even m: x0 + x_{I/2} +- u_Q (re), 0 (im); odd m: x0 - x_{I/2} (re),
    // +- v_Q (im); the sign is (-1)^p, p = 8 pg + q
    float acc[8][8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const float4 b = b0s[8 * rg + r];
      const float e0 = b.x + b.y;
      float v0, v1;                            // q even, q odd
      if (c == 0) { v0 = e0 + b.z; v1 = e0 - b.z; }
      else if (c == 1) { v0 = 0.f; v1 = 0.f; }
      else if (c == 2) { v0 = b.x - b.y; v1 = v0; }
      else { v0 = b.w; v1 = -b.w; }
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[r][q] = (q & 1) ? v1 : v0;
    }
    if (active) {
      const float* pa = pln + c * PS + 8 * rg;
      const float* pt = tab + c * TS + 8 * pg;
#pragma unroll 2
      for (int i = 1; i < Q; ++i) {
        const float4 a0 = *reinterpret_cast<const float4*>(pa + i * RP);
        const float4 a1 = *reinterpret_cast<const float4*>(pa + i * RP + 4);
        const float4 t0 = *reinterpret_cast<const float4*>(pt + i * NPP);
        const float4 t1 = *reinterpret_cast<const float4*>(pt + i * NPP + 4);
        const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float tv[8] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w};
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
          for (int q = 0; q < 8; ++q) acc[r][q] = fmaf(av[r], tv[q], acc[r][q]);
      }
    }
    __syncthreads();                         // planes read: the staged outputs overwrite them

    // Epilogue.  Quarters 0 and 1 (2 and 3) hold the real and imaginary sums
    // of even (odd) m for the same tile; partners exchange half their pairs
    // so that each holds X = (S_re, -S_im) of 8 rows by 4 pairs: the even
    // quarter pairs 0-3 of its group, the odd quarter pairs 4-7.  A level's
    // group gives its six fields (a3 = wg X(gt) - wd i m X(xu), a5 from g,
    // yu; fu fv ke xv); the trailing groups give yv and the surface rows.
    const float gw = d.jfac[JF_GW * J + j], gwdc = d.jfac[JF_GWDELC * J + j];
    const float wg = gw / float(I), wd = gwdc / float(I);
    float2* fo = reinterpret_cast<float2*>(pln);     // [M][7 lc]: item m lc + l at 7 (m lc + l)
    const bool ev = (c & 1) == 0;
    const int par = c >> 1;                          // 0: even m, 1: odd m
    const int NP = (M + 1) >> 1;
#pragma unroll
    for (int rp = 0; rp < 4; ++rp) {
      float re[2][4], im[2][4];
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float send = ev ? acc[2 * rp + h][4 + q] : acc[2 * rp + h][q];
          const float recv = __shfl_xor_sync(0xffffffffu, send, 8);
          re[h][q] = ev ? acc[2 * rp + h][q] : recv;
          im[h][q] = ev ? recv : acc[2 * rp + h][4 + q];
        }
      if (!active) continue;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int p = 8 * pg + (ev ? 0 : 4) + q, m = 2 * p + par;
        if (p >= NP || m >= M) continue;
        // X_h = (re[h], -im[h])
        if (rg < lc) {
          float2* o = fo + AF_N * (m * lc + rg);
          const float wdm = wd * float(m);
          if (rp < 2) {
            // rows (gt, xu) or (g, yu): wg X0 - wd i m X1
            o[rp == 0 ? AF_T : AF_Q] = make_float2(wg * re[0][q] + wdm * -im[1][q],
                                                   wg * -im[0][q] - wdm * re[1][q]);
          } else if (rp == 2) {
            o[AF_FU] = make_float2(wd * re[0][q], wd * -im[0][q]);
            o[AF_FV] = make_float2(wd * re[1][q], wd * -im[1][q]);
          } else {
            o[AF_KE] = make_float2(wg * re[0][q], wg * -im[0][q]);
            o[AF_XV] = make_float2(wd * re[1][q], wd * -im[1][q]);
          }
        } else {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int pr = 8 * rg + 2 * rp + h;
            if (pr < 9 * lc) {
              fo[AF_N * (m * lc + (pr - 8 * lc)) + AF_YV] = make_float2(wd * re[h][q], wd * -im[h][q]);
            } else if (surf && pr < 9 * lc + 2) {
              float2* os = reinterpret_cast<float2*>(d.afs);
              os[(((size_t)e * M + m) * J + j) * 2 + (pr - 9 * lc)] =
                  make_float2(wg * re[h][q], wg * -im[h][q]);
            }
          }
        }
      }
    }
    const int nitem = M * lc;
    __syncthreads();
    {
      // staged rows -> af, consecutive threads on consecutive addresses
      const int RS = AF_N * lc;
      const unsigned mg = (unsigned)((0x100000000ull + RS - 1) / RS);   // y / RS, y < 2^16
      float2* afu = reinterpret_cast<float2*>(d.af) + (((size_t)e * M * J + j) * K + k0) * AF_N;
      const size_t mstride = (size_t)J * K * AF_N;
      for (int y = tid; y < AF_N * nitem; y += nt) {
        const int m = __umulhi((unsigned)y, mg);
        afu[m * mstride + (y - m * RS)] = fo[y];
      }
    }
  }
}

}  // namespace lbm
