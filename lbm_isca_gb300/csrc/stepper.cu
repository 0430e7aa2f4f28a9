// Fused ensemble stepper: the per-step hot path of LBM.run
// (model.py:213-247) for many members at once, with the prognostic state in
// packed spectral space.
//
// One step = four launches:
//   k_grid      per (member, latitude): inverse FFTs of the synthesised
//               Fourier fields, the whole grid-point tendency algebra of
//               dynamics.py:176-262 level by level, forward FFTs, weighting;
//               also the grid-space Robert-Asselin filter of ps (state.py
//               :110-128 acts on ps, which is nonlinear in pi).
//   k_anal      per (member, m-pair, level chunk): Legendre analysis with the
//               equatorial symmetry split -> explicit spectral tendencies.
//   k_implicit  per (member, n-pair): semi-implicit solve, leapfrog, implicit
//               damping / vertical diffusion, spectral Robert-Asselin filter
//               (integrator.py:264-315, state.py:110-128), column sums.
//   k_synth     per (member, m-pair, level chunk): Legendre synthesis of the
//               new level -> Fourier fields for the next k_grid.
//
// The reference keeps its state in grid space; u, v, T, q are band-limited,
// so filtering and advancing them in spectral space is exact to round-off.
// ps is not band-limited after its filter, so its two grid levels are kept.
// The column sum of dsig*(div + v.grad ln ps) that defines sigma-dot is
// split into its linear parts, which are synthesised from sigma-weighted
// column sums of psi, chi and div computed in k_implicit; k_grid then needs
// no second pass over the levels.
#include "lbm_common.cuh"
#include "lbm_fft.cuh"
#include "async_copy.cuh"
#include <cmath>
#include <mutex>
#include <new>
#include <type_traits>

namespace lbm {

// ---- typed view of the descriptor ---------------------------------------------
template <typename R> struct SD {
  int E, J, I, N, M, K, NS, nsets, strictly_linear, frc_shared;
  int vd_on[4];
  R kappa, epsvt, robert;
  const R *symp, *symh;
  const C2<R>* tw;
  const R *jfac, *vert, *b3, *bsd, *b2;
  const R *lap, *invlap, *nn1a, *kv, *kd, *ktt, *kq, *ww, *tmtx, *minv, *vdiff;
  const C2<R> *frc3, *frcs;
  const float2* dft;
  C2<R> *sa3, *sas, *sb3;
  R *psa, *psb;
  C2<R> *sf, *sfs, *af, *afs, *tend, *tends;
  float *grid6, *grid9;
  int* err;
  int* err_member;
  int legendre;                          // 0 FMA; 3 or 6: tensor-core products
  const unsigned char* tc_anal;          // table image of k_anal_tc
  const unsigned char* tc_synth;         // table image of k_synth_tc
  int tc_off;                            // bits 0 / 1 / 2: Legendre analysis / synthesis,
                                         // longitude analysis on FMA
  int tc_g;                              // members per MMA tile cap (0: as many as fit)
  const unsigned char* tc_dft;           // table image of k_fdft_tc
};

template <typename R> SD<R> make_sd(const lbm_stepper_desc& d) {
  SD<R> s;
  s.E = d.nmem; s.J = d.nlat; s.I = d.nlon; s.N = d.nmax; s.M = d.nmax + 1; s.K = d.kmax;
  s.NS = nspec(d.nmax); s.nsets = d.nsets; s.strictly_linear = d.strictly_linear;
  s.frc_shared = d.frc_shared;
  for (int i = 0; i < 4; ++i) s.vd_on[i] = d.vd_on[i];
  s.kappa = R(d.kappa); s.epsvt = R(d.epsvt); s.robert = R(d.robert);
  s.symp = (const R*)d.symp; s.symh = (const R*)d.symh; s.tw = (const C2<R>*)d.tw;
  s.jfac = (const R*)d.jfac; s.vert = (const R*)d.vert; s.b3 = (const R*)d.b3;
  s.bsd = (const R*)d.bsd; s.b2 = (const R*)d.b2;
  s.lap = (const R*)d.lap; s.invlap = (const R*)d.invlap; s.nn1a = (const R*)d.nn1a;
  s.kv = (const R*)d.kv; s.kd = (const R*)d.kd; s.ktt = (const R*)d.ktt; s.kq = (const R*)d.kq;
  s.ww = (const R*)d.ww; s.tmtx = (const R*)d.tmtx; s.minv = (const R*)d.minv;
  s.vdiff = (const R*)d.vdiff;
  s.frc3 = (const C2<R>*)d.frc3; s.frcs = (const C2<R>*)d.frcs;
  s.dft = (const float2*)d.dft;
  s.sa3 = (C2<R>*)d.sa3; s.sas = (C2<R>*)d.sas; s.sb3 = (C2<R>*)d.sb3;
  s.psa = (R*)d.psa; s.psb = (R*)d.psb;
  s.sf = (C2<R>*)d.sf; s.sfs = (C2<R>*)d.sfs; s.af = (C2<R>*)d.af; s.afs = (C2<R>*)d.afs;
  s.tend = (C2<R>*)d.tend; s.tends = (C2<R>*)d.tends;
  s.grid6 = (float*)d.grid6; s.grid9 = (float*)d.grid9;
  s.err = d.err;
  s.err_member = d.err_member;
  s.legendre = d.legendre;
  s.tc_anal = (const unsigned char*)d.tc_anal;
  s.tc_synth = (const unsigned char*)d.tc_synth;
  s.tc_off = d.tc_off;
  s.tc_g = d.tc_g;
  s.tc_dft = (const unsigned char*)d.tc_dft;
  return s;
}

// basic-state 3-D field indices in b3 [10][J][K][I]
enum { B_U = 0, B_V, B_T, B_Q, B_TV, B_ABSVOR, B_DIV, B_X5, B_TDEV, B_TVDEV,
       B_HDU, B_HDV, B_HDT, B_HDQ, B_N };
// b2 [5][J][I]
enum { B2_PIX = 0, B2_PIY, B2_PSBAR, B2_USUM, B2_VSUM };
// jfac [4][J]
enum { JF_GW = 0, JF_GWDELC, JF_RCOS, JF_COS };
// Fourier field slots
enum { SF_U = 0, SF_V, SF_VOR, SF_DIV, SF_T, SF_Q, SF_N };           // sf [..][6]
enum { SFS_PI = 0, SFS_PIY, SFS_UH, SFS_VH, SFS_DH, SFS_N };         // sfs [..][5]
enum { AF_FU = 0, AF_FV, AF_KE, AF_T, AF_XV, AF_Q, AF_YV, AF_N };     // af [..][7]

template <typename R> LBM_D R vrow(const SD<R>& d, int row, int k) {
  return d.vert[row * (d.K + 1) + k];
}

// =============================================================================
// k_grid: Fourier -> grid -> tendency algebra -> Fourier, per (member, lat)
// =============================================================================
template <typename R, int I, int KB, int NT> struct GridSmem {
  static constexpr int R1 = FftShape<I>::R1;
  static constexpr int NTEAM = NT / R1;
  static constexpr int SCR = fft_team_scratch<I>();
  static constexpr int RS = KB + 2;          // ring slots of grid levels
  static constexpr int NG = 9;               // grid outputs per level
  static constexpr int NIN = (KB + 1) * SF_N;   // Fourier staging in (levels)
  static constexpr int NOUT = KB * AF_N;         // Fourier staging out
  static size_t bytes(int M) {
    return sizeof(C2<R>) * (size_t)(I + NTEAM * SCR + (NIN + NOUT) * M) +
           sizeof(R) * (size_t)I * (RS * SF_N + KB * NG + KB * 5 + 8 + 3);
  }
};

template <typename R> LBM_D R vadv(R fm, R f0, R fp, R s0, R s1, bool lo, bool hi, R dsk) {
  const R flo = lo ? s0 * R(0.5) * (f0 + fm) : R(0);
  const R fhi = hi ? s1 * R(0.5) * (fp + f0) : R(0);
  return (fhi - flo - f0 * (s1 - s0)) / dsk;
}

template <typename R, int I, int KB, int NT>
__global__ void __launch_bounds__(NT) k_grid(SD<R> d, int ps_mode) {
  using SM = GridSmem<R, I, KB, NT>;
  constexpr int R1 = SM::R1, NTEAM = SM::NTEAM, SCR = SM::SCR, RS = SM::RS, NG = SM::NG;
  const int j = blockIdx.x, e = blockIdx.y;
  const int J = d.J, K = d.K, M = d.M;
  const int tid = threadIdx.x, team = tid / R1, t = tid % R1;
  extern __shared__ unsigned char smraw[];
  C2<R>* tw = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* scr = tw + I;
  C2<R>* fin = scr + NTEAM * SCR;                     // [KB+1][6][M] (or [5][M])
  C2<R>* fout = fin + SM::NIN * M;                     // [KB][7][M] (or [2][M])
  R* gin = reinterpret_cast<R*>(fout + SM::NOUT * M);  // [RS][6][I]
  R* gout = gin + RS * SF_N * I;                       // [KB][9][I]
  R* pre = gout + KB * NG * I;                         // [KB][5][I]
  R* sg = pre + KB * 5 * I;                            // [8][I] surface fields
  R* pst = sg + 8 * I;                                 // [3][I] running column prefixes
  for (int c = tid; c < I; c += NT) pst[c] = pst[I + c] = pst[2 * I + c] = R(0);

  for (int p = tid; p < I; p += NT) tw[p] = d.tw[p];
  const R gw = d.jfac[JF_GW * J + j], gwdc = d.jfac[JF_GWDELC * J + j];
  const R rcos = d.jfac[JF_RCOS * J + j];
  const R invI = R(1) / R(I);
  const size_t jmK = (size_t)J * K;
  const C2<R>* sfe = d.sf + (size_t)e * M * jmK * SF_N;
  C2<R>* afe = d.af + (size_t)e * M * jmK * AF_N;

  // ---- surface pre-pass ----------------------------------------------------
  for (int idx = tid; idx < M * SFS_N; idx += NT) {
    const int m = idx / SFS_N, f = idx % SFS_N;
    fin[f * M + m] = d.sfs[(((size_t)e * M + m) * J + j) * SFS_N + f];
  }
  __syncthreads();
  // jobs: 0 pi, 1 pi_x (i m pi, /(a cos)), 2 pi_y, 3 U-sum, 4 V-sum, 5 D-sum
  for (int job = team; job < 6; job += NTEAM) {
    const int src = (job <= 1) ? SFS_PI : job - 1;   // PI, PI, PIY, UH, VH, DH
    const C2<R>* X = fin + src * M;
    const R sc = (job == 0 || job == 5) ? R(1) : rcos;
    if (job == 1)
      team_rfft_inv<I>(t, [&](int m) { return im_mul(X[m], R(m)); }, M, scr + team * SCR, tw,
                       sg + job * I, 1, sc);
    else
      team_rfft_inv<I>(t, [&](int m) { return X[m]; }, M, scr + team * SCR, tw, sg + job * I,
                       1, sc);
  }
  __syncthreads();
  // per column: total column sum S_tot, gt_pi, ps update, pi(t - dt)
  const R* b2 = d.b2;
  for (int c = tid; c < I; c += NT) {
    const size_t g2 = (size_t)j * I + c;
    const R pixb = b2[(B2_PIX * J) * I + g2], piyb = b2[(B2_PIY * J) * I + g2];
    const R psbar = b2[(B2_PSBAR * J) * I + g2];
    const R usum = b2[(B2_USUM * J) * I + g2], vsum = b2[(B2_VSUM * J) * I + g2];
    const R pi = sg[0 * I + c], pix = sg[1 * I + c], piy = sg[2 * I + c];
    const R uh = sg[3 * I + c], vh = sg[4 * I + c], dh = sg[5 * I + c];
    const R stot = dh + pixb * uh + piyb * vh + pix * usum + piy * vsum;
    sg[6 * I + c] = stot;
    sg[7 * I + c] = dh;
    gout[0 * I + c] = dh - stot;                 // gt_pi (dynamics.py:188)
    const size_t gp = (size_t)e * J * I + g2;
    const R pscur = psbar * expm1(pi);           // state.py:81-83
    R pb = d.psb[gp];
    if (ps_mode == 1) {
      pb = d.psa[gp];
    } else if (ps_mode == 2) {
      const R pa = d.psa[gp];
      pb = pa + d.robert * (pb - R(2) * pa + pscur);
    }
    if (ps_mode != 0) {
      d.psb[gp] = pb;
      d.psa[gp] = pscur;
    }
    gout[1 * I + c] = log1p(pb / psbar);         // pi' of the filtered t - dt level
  }
  __syncthreads();
  for (int job = team; job < 2; job += NTEAM) {
    C2<R>* Y = fout + job * M;
    team_rfft_fwd<I>(t, gout + job * I, 1, scr + team * SCR, tw, M, gw * invI,
                     [&](int m, C2<R> X) { Y[m] = X; });
  }
  __syncthreads();
  for (int idx = tid; idx < M * 2; idx += NT) {
    const int m = idx / 2, f = idx % 2;
    d.afs[(((size_t)e * M + m) * J + j) * 2 + f] = fout[f * M + m];
  }

  // ---- level loop -----------------------------------------------------------
  const R eps = d.epsvt, kappa = d.kappa;
  const R* b3 = d.b3;
  auto B3 = [&](int f, int k, int c) -> R { return b3[(((size_t)f * J + j) * K + k) * I + c]; };
  auto BSD = [&](int k, int c) -> R { return d.bsd[((size_t)j * (K + 1) + k) * I + c]; };
  auto GIN = [&](int k, int f) -> R* { return gin + ((k % RS) * SF_N + f) * I; };

  for (int k0 = 0; k0 < K; k0 += KB) {
    const int lo = (k0 == 0) ? 0 : k0 + 1;
    const int hi = min(k0 + KB, K - 1);
    const int nl = hi - lo + 1;                 // levels to load (may be 0)
    __syncthreads();
    if (nl > 0) {
      for (int idx = tid; idx < M * nl * SF_N; idx += NT) {
        const int m = idx / (nl * SF_N), r = idx % (nl * SF_N);
        const int l = r / SF_N, f = r % SF_N;
        fin[(l * SF_N + f) * M + m] = sfe[((size_t)m * J + j) * K * SF_N + (size_t)(lo + l) * SF_N + f];
      }
      __syncthreads();
      for (int job = team; job < nl * SF_N; job += NTEAM) {
        const int l = job / SF_N, f = job % SF_N;
        const C2<R>* X = fin + (l * SF_N + f) * M;
        const R sc = (f == SF_U || f == SF_V) ? rcos : R(1);
        team_rfft_inv<I>(t, [&](int m) { return X[m]; }, M, scr + team * SCR, tw,
                         GIN(lo + l, f), 1, sc);
      }
      __syncthreads();
    }
    const int kb = min(KB, K - k0);             // levels processed this iteration
    // column prefixes (one thread per column, levels in order)
    for (int c = tid; c < I; c += NT) {
      const size_t g2 = (size_t)j * I + c;
      const R pixb = b2[(B2_PIX * J) * I + g2], piyb = b2[(B2_PIY * J) * I + g2];
      const R pix = sg[1 * I + c], piy = sg[2 * I + c], stot = sg[6 * I + c],
              dh = sg[7 * I + c];
      R pref = pst[c], prefd = pst[I + c], pref3 = pst[2 * I + c];
      for (int l = 0; l < kb; ++l) {
        const int k = k0 + l;
        const R u = GIN(k, SF_U)[c], v = GIN(k, SF_V)[c], dv = GIN(k, SF_DIV)[c];
        const R tt = GIN(k, SF_T)[c], q = GIN(k, SF_Q)[c];
        const R padv = u * pixb + B3(B_U, k, c) * pix + v * piyb + B3(B_V, k, c) * piy;
        R* pr = pre + (l * 5) * I;
        pr[0 * I + c] = stot - pref;                       // S[k]
        pref += (dv + padv) * vrow(d, LBM_VERT_DSIG, k);
        pr[1 * I + c] = stot - pref;                       // S[k+1]
        prefd += dv * vrow(d, LBM_VERT_DSIG, k);
        pr[2 * I + c] = dh - prefd;                        // sum_{l>k} dsig div
        const R x = eps * (tt * B3(B_Q, k, c) + B3(B_T, k, c) * q);   // Tv' - T'
        pr[3 * I + c] = pref3 + vrow(d, LBM_VERT_RALPHA, k) * x;      // (WW x)_k
        pref3 += vrow(d, LBM_VERT_RDLOG3, k) * x;
        pr[4 * I + c] = padv;
      }
      pst[c] = pref;
      pst[I + c] = prefd;
      pst[2 * I + c] = pref3;
    }
    __syncthreads();
    // pointwise algebra, (level, column) per thread
    for (int it = tid; it < kb * I; it += NT) {
      const int l = it / I, c = it % I, k = k0 + l;
      const size_t g2 = (size_t)j * I + c;
      const R pixb = b2[(B2_PIX * J) * I + g2], piyb = b2[(B2_PIY * J) * I + g2];
      const R pix = sg[1 * I + c], piy = sg[2 * I + c], stot = sg[6 * I + c];
      const R* pr = pre + (l * 5) * I;
      const R S0 = pr[0 * I + c], S1 = pr[1 * I + c], sdv = pr[2 * I + c];
      const R phiv = pr[3 * I + c], padv = pr[4 * I + c];
      const bool hasm = k >= 1, hasp = k + 1 <= K - 1;
      const int km = hasm ? k - 1 : k, kp = hasp ? k + 1 : k;
      const R sd0 = hasm ? vrow(d, LBM_VERT_SIGM, k) * stot - S0 : R(0);
      const R sd1 = hasp ? vrow(d, LBM_VERT_SIGM, k + 1) * stot - S1 : R(0);
      const R sb0 = BSD(k, c), sb1 = BSD(k + 1, c);
      const R dsk = vrow(d, LBM_VERT_DSIG, k);
      const R u = GIN(k, SF_U)[c], v = GIN(k, SF_V)[c], vo = GIN(k, SF_VOR)[c];
      const R dv = GIN(k, SF_DIV)[c], tt = GIN(k, SF_T)[c], q = GIN(k, SF_Q)[c];
      const R ub = B3(B_U, k, c), vb = B3(B_V, k, c), tb = B3(B_T, k, c), qb = B3(B_Q, k, c);
      const R tvb = B3(B_TV, k, c), absv = B3(B_ABSVOR, k, c), divb = B3(B_DIV, k, c);
      const R x5b = B3(B_X5, k, c), tdev = B3(B_TDEV, k, c), tvdev = B3(B_TVDEV, k, c);
      const R tv = tt + eps * (tt * qb + tb * q);
      const R x5p = vrow(d, LBM_VERT_ALPHA, k) * dv + vrow(d, LBM_VERT_WP, k) * padv +
                    vrow(d, LBM_VERT_W3, k) * S1;
      const R adiab = -kappa * (tv * x5b + tvb * x5p);
      const R hadv = tt * divb + tdev * dv;
      const R vadvT = vadv(GIN(km, SF_T)[c], tt, GIN(kp, SF_T)[c], sb0, sb1, hasm, hasp, dsk) +
                      vadv(B3(B_T, km, c), tb, B3(B_T, kp, c), sd0, sd1, hasm, hasp, dsk);
      const R tm = vrow(d, LBM_VERT_KTREF, k) *
                   (vrow(d, LBM_VERT_ALPHA, k) * dv + vrow(d, LBM_VERT_W3, k) * sdv);
      R* go = gout + (l * NG) * I;
      go[3 * I + c] = adiab + hadv + vadvT + tm;                          // gt_t
      go[4 * I + c] = u * tdev + ub * tt;                                 // xu
      go[5 * I + c] = v * tdev + vb * tt;                                 // xv
      const R rcpg = vrow(d, LBM_VERT_RCPG, k);
      R fu = v * absv + vb * vo - rcpg * (tv * pixb + tvdev * pix);
      R fv = -u * absv - ub * vo - rcpg * (tv * piyb + tvdev * piy);
      fu += vadv(GIN(km, SF_U)[c], u, GIN(kp, SF_U)[c], sb0, sb1, hasm, hasp, dsk) +
            vadv(B3(B_U, km, c), ub, B3(B_U, kp, c), sd0, sd1, hasm, hasp, dsk);
      fv += vadv(GIN(km, SF_V)[c], v, GIN(kp, SF_V)[c], sb0, sb1, hasm, hasp, dsk) +
            vadv(B3(B_V, km, c), vb, B3(B_V, kp, c), sd0, sd1, hasm, hasp, dsk);
      go[0 * I + c] = fu;
      go[1 * I + c] = fv;
      R ke = phiv + u * ub + v * vb;
      if (!d.strictly_linear) ke += R(0.5) * (u * u + v * v);
      go[2 * I + c] = ke;
      go[6 * I + c] = q * divb + qb * dv +
                      vadv(GIN(km, SF_Q)[c], q, GIN(kp, SF_Q)[c], sb0, sb1, hasm, hasp, dsk) +
                      vadv(B3(B_Q, km, c), qb, B3(B_Q, kp, c), sd0, sd1, hasm, hasp, dsk);
      go[7 * I + c] = u * qb + ub * q;                                    // yu
      go[8 * I + c] = v * qb + vb * q;                                    // yv
    }
    __syncthreads();
    // forward FFTs, weighted and combined into the 7 analysis inputs
    const R wd = gwdc * invI, wg = gw * invI;
    for (int job = team; job < kb * AF_N; job += NTEAM) {
      const int l = job / AF_N, a = job % AF_N;
      const R* go = gout + (l * NG) * I;
      C2<R>* Y = fout + (l * AF_N + a) * M;
      C2<R>* sc_ = scr + team * SCR;
      switch (a) {
        case AF_FU: team_rfft_fwd<I>(t, go + 0 * I, 1, sc_, tw, M, wd, [&](int m, C2<R> X) { Y[m] = X; }); break;
        case AF_FV: team_rfft_fwd<I>(t, go + 1 * I, 1, sc_, tw, M, wd, [&](int m, C2<R> X) { Y[m] = X; }); break;
        case AF_KE: team_rfft_fwd<I>(t, go + 2 * I, 1, sc_, tw, M, wg, [&](int m, C2<R> X) { Y[m] = X; }); break;
        case AF_T:
          team_rfft_fwd<I>(t, go + 3 * I, 1, sc_, tw, M, wg, [&](int m, C2<R> X) { Y[m] = X; });
          team_rfft_fwd<I>(t, go + 4 * I, 1, sc_, tw, M, wd,
                           [&](int m, C2<R> X) { Y[m] = Y[m] - im_mul(X, R(m)); });
          break;
        case AF_XV: team_rfft_fwd<I>(t, go + 5 * I, 1, sc_, tw, M, wd, [&](int m, C2<R> X) { Y[m] = X; }); break;
        case AF_Q:
          team_rfft_fwd<I>(t, go + 6 * I, 1, sc_, tw, M, wg, [&](int m, C2<R> X) { Y[m] = X; });
          team_rfft_fwd<I>(t, go + 7 * I, 1, sc_, tw, M, wd,
                           [&](int m, C2<R> X) { Y[m] = Y[m] - im_mul(X, R(m)); });
          break;
        default: team_rfft_fwd<I>(t, go + 8 * I, 1, sc_, tw, M, wd, [&](int m, C2<R> X) { Y[m] = X; }); break;
      }
    }
    __syncthreads();
    for (int idx = tid; idx < M * kb * AF_N; idx += NT) {
      const int m = idx / (kb * AF_N), r = idx % (kb * AF_N);
      const int l = r / AF_N, a = r % AF_N;
      afe[((size_t)m * J + j) * K * AF_N + (size_t)(k0 + l) * AF_N + a] = fout[(l * AF_N + a) * M + m];
    }
  }
}

// =============================================================================
// Legendre analysis: af -> tend, per (member, m-pair, level chunk)
// =============================================================================
constexpr int AN_JC = 8;      // latitude pairs staged per pass

template <typename R> struct PairRows {
  int m1, m2, L1, L2, NR;
  LBM_D PairRows(int p, int N) {
    m1 = p;
    m2 = N - p;
    L1 = N + 1 - m1;
    L2 = (m2 != m1) ? N + 1 - m2 : 0;
    NR = L1 + L2;
  }
  LBM_D int m_of(int r) const { return r < L1 ? m1 : m2; }
  LBM_D int n_of(int r) const { return r < L1 ? m1 + r : m2 + (r - L1); }
};

// Row groups of the analysis block: NC rows of an m-pair's N + 2 (at most
// two partial groups).
template <int NC> LBM_HD int anal_groups(int N) { return (N + 2 + NC - 1) / NC + 1; }

// Members per block of the surface-only forms (one table staging serves them).
constexpr int SURF_EB = 16;

// SURF: only the surface part (tends), for the tensor-core analysis, which
// computes the level part (k_anal_tc).
template <typename R, int NC, int KC, bool SURF = false>
__global__ void k_anal(SD<R> d) {
  const int p = blockIdx.x, e = blockIdx.y, kc = blockIdx.z;
  const int J = d.J, K = d.K, N = d.N, M = d.M, JH = J / 2;
  const int k0 = kc * KC, kn = min(KC, K - k0);
  const PairRows<R> pr(p, N);
  const int G1 = (pr.L1 + NC - 1) / NC, G2 = (pr.L2 + NC - 1) / NC;
  const int G = anal_groups<NC>(N);                    // row groups of the block
  const int TS = NC * G + 1;                           // odd latitude stride of the tables
  extern __shared__ unsigned char smraw[];
  // P and H of the pair's rows as [JH][NC][G]: row rbase(g) + i at slot i G + g,
  // so the row groups of a warp read adjacent words (no bank conflict)
  R* tp = reinterpret_cast<R*>(smraw);
  R* th = tp + (size_t)JH * TS;
  // rows of AN_JC latitude pairs, two buffers, each
  // [2 m][AN_JC][2 hemispheres][KC levels][7 fields] (16-byte aligned)
  C2<R>* raw = reinterpret_cast<C2<R>*>(
      (reinterpret_cast<uintptr_t>(th + (size_t)JH * TS) + 15) & ~uintptr_t(15));
  const int tid = threadIdx.x, nt = blockDim.x;
  const int off1 = spec_offset(pr.m1, N), off2 = spec_offset(pr.m2, N);
  {
    const FastDiv fjh(JH), fg(G);
    for (int idx = tid; idx < NC * G * JH; idx += nt) {
      const int sl = fjh.div(idx), jh = idx - sl * JH;     // latitude fastest
      const int i = fg.div(sl), gg = sl - i * G;
      int row = -1;
      if (gg < G1) {
        const int r = gg * NC + i;
        if (r < pr.L1) row = off1 + r;
      } else if (gg < G1 + G2) {
        const int r = (gg - G1) * NC + i;
        if (r < pr.L2) row = off2 + r;
      }
      tp[jh * TS + sl] = row >= 0 ? d.symp[(size_t)row * JH + jh] : R(0);
      th[jh * TS + sl] = row >= 0 ? d.symh[(size_t)row * JH + jh] : R(0);
    }
  }
  const int nm = pr.L2 ? 2 : 1;
  if constexpr (!SURF) {
  const int k = tid % KC, g = tid / KC;
  const bool active = (k < kn) && (g < G1 + G2);
  const int mi = (g < G1) ? 0 : 1;
  const int rbase = (g < G1) ? g * NC : pr.L1 + (g - G1) * NC;
  const int rend = (g < G1) ? pr.L1 : pr.NR;
  C2<R> acc[NC][9];
#pragma unroll
  for (int i = 0; i < NC; ++i)
#pragma unroll
    for (int a = 0; a < 9; ++a) acc[i][a] = cmk<R>(0, 0);
  const size_t jmK = (size_t)J * K;
  const C2<R>* afe = d.af + (size_t)e * M * jmK * AF_N;
  const int rowlen = kn * AF_N;                 // complex values per (m, latitude) row
  const int rowst = KC * AF_N;                  // row stride in the buffer
  const size_t rawbuf = (size_t)2 * AN_JC * 2 * rowst;
  // 16-byte copies when every row starts and ends on a 16-byte boundary
  constexpr int PER = 16 / (int)sizeof(C2<R>);
  const bool wide = ((K * AF_N) % PER == 0) && ((k0 * AF_N) % PER == 0) &&
                    (rowlen % PER == 0) && (rowst % PER == 0);
  const int step = wide ? PER : 1;
  const int nchunk = rowlen / step;
  const FastDiv fch(nchunk);
  auto prefetch = [&](int jh0, int b) {
    const int jc = min(AN_JC, JH - jh0);
    C2<R>* rb = raw + b * rawbuf;
    // rows w = (mm AN_JC + jj) 2 + hemi; those with jj >= jc are skipped
    for (int x = tid; x < nm * AN_JC * 2 * nchunk; x += nt) {
      const int w = fch.div(x), c = (x - w * nchunk) * step;
      const int hemi = w & 1, jj = (w >> 1) & (AN_JC - 1), mm = w / (2 * AN_JC);
      if (jj >= jc) continue;
      const int m = mm ? pr.m2 : pr.m1;
      const int jn = jh0 + jj, j = hemi ? J - 1 - jn : jn;
      C2<R>* dst = rb + ((mm * AN_JC + jj) * 2 + hemi) * rowst + c;
      const C2<R>* src = afe + (((size_t)m * J + j) * K + k0) * AF_N + c;
      if (wide) cp_async16(dst, src);
      else cp_async_c2(dst, src);
    }
    cp_async_commit();
  };
  prefetch(0, 0);
  int buf = 0;
  for (int jh0 = 0; jh0 < JH; jh0 += AN_JC) {
    const int jc = min(AN_JC, JH - jh0);
    if (jh0 + AN_JC < JH) prefetch(jh0 + AN_JC, buf ^ 1);
    else cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    if (active) {
      const C2<R>* rb = raw + buf * rawbuf;
      for (int jj = 0; jj < jc; ++jj) {
        // north / south rows -> equatorially symmetric [0] and antisymmetric [1] parts
        const C2<R>* xn = rb + ((mi * AN_JC + jj) * 2) * rowst + k * AF_N;
        const C2<R>* xsth = xn + rowst;
        C2<R> x[AF_N][2];
#pragma unroll
        for (int f = 0; f < AF_N; ++f) {
          const C2<R> a = xn[f], b = xsth[f];
          x[f][0] = a + b;
          x[f][1] = a - b;
        }
        const int jh = jh0 + jj;
#pragma unroll
        for (int i = 0; i < NC; ++i) {
          const int r = rbase + i;
          if (r >= rend) break;
          const R P = tp[jh * TS + i * G + g], H = th[jh * TS + i * G + g];
          const int ps = (i & 1);          // parity of (n - m): rows alternate
          const int hs = ps ^ 1;
          cfma(acc[i][0], P, x[AF_FU][ps]);
          cfma(acc[i][1], P, x[AF_FV][ps]);
          cfma(acc[i][2], P, x[AF_KE][ps]);
          cfma(acc[i][3], P, x[AF_T][ps]);
          cfma(acc[i][4], P, x[AF_Q][ps]);
          cfma(acc[i][5], H, x[AF_FU][hs]);
          cfma(acc[i][6], H, x[AF_FV][hs]);
          cfma(acc[i][7], H, x[AF_XV][hs]);
          cfma(acc[i][8], H, x[AF_YV][hs]);
        }
      }
    }
    buf ^= 1;
    __syncthreads();
  }
  if (active) {
    const size_t NS = d.NS;
#pragma unroll
    for (int i = 0; i < NC; ++i) {
      const int r = rbase + i;
      if (r >= rend) break;
      const int m = pr.m_of(r), n = pr.n_of(r);
      const size_t idx = (size_t)spec_index(m, n, N);
      const R rm = R(m);
      const C2<R> vor = im_mul(acc[i][1], rm) + acc[i][5];
      const C2<R> div = im_mul(acc[i][0], rm) - acc[i][6] + acc[i][2] * d.nn1a[n];
      const C2<R> tt = acc[i][3] + acc[i][7];
      const C2<R> qq = acc[i][4] + acc[i][8];
      C2<R>* te = d.tend + (size_t)e * 4 * NS * K;
      te[(0 * NS + idx) * K + k0 + k] = vor;
      te[(1 * NS + idx) * K + k0 + k] = div;
      te[(2 * NS + idx) * K + k0 + k] = tt;
      te[(3 * NS + idx) * K + k0 + k] = qq;
    }
  }
  }  // !SURF
  // surface: wt_pi and pi(t - dt), one thread per row (first level chunk
  // only; the surface-only form takes SURF_EB members per block)
  auto surface = [&](int e) {
  __syncthreads();
  C2<R>* ss = raw;                                   // [2][JH][2 fields][2]
  for (int idx = tid; idx < nm * JH * 2; idx += nt) {
    const int f = idx % 2, jh = (idx / 2) % JH, mm = idx / (2 * JH);
    const int m = mm ? pr.m2 : pr.m1;
    const C2<R> xn = d.afs[(((size_t)e * M + m) * J + jh) * 2 + f];
    const C2<R> xsouth = d.afs[(((size_t)e * M + m) * J + (J - 1 - jh)) * 2 + f];
    C2<R>* dst = ss + ((mm * JH + jh) * 2 + f) * 2;
    dst[0] = xn + xsouth;
    dst[1] = xn - xsouth;
  }
  __syncthreads();
  for (int r = tid; r < pr.NR; r += nt) {
    const int m = pr.m_of(r), n = pr.n_of(r), mm = r < pr.L1 ? 0 : 1;
    const int par = (n - m) & 1;
    C2<R> a0 = cmk<R>(0, 0), a1 = cmk<R>(0, 0);
    const int rr = r < pr.L1 ? r : r - pr.L1;
    const int sl = (rr % NC) * G + (r < pr.L1 ? 0 : G1) + rr / NC;   // table slot of row r
    for (int jh = 0; jh < JH; ++jh) {
      const R P = tp[jh * TS + sl];
      const C2<R>* x = ss + ((mm * JH + jh) * 2) * 2;
      cfma(a0, P, x[0 * 2 + par]);
      cfma(a1, P, x[1 * 2 + par]);
    }
    const size_t idx = (size_t)spec_index(m, n, N);
    d.tends[((size_t)e * 2 + 0) * d.NS + idx] = a0;
    d.tends[((size_t)e * 2 + 1) * d.NS + idx] = a1;
  }
  };
  if constexpr (SURF) {
    const int e1 = min(d.E, (int)(blockIdx.y + 1) * SURF_EB);
    for (int ee = blockIdx.y * SURF_EB; ee < e1; ++ee) surface(ee);
  } else {
    if (kc != 0) return;
    surface(e);
  }
}

// =============================================================================
// Implicit spectral update, per (member, n-pair)
// =============================================================================
constexpr int IM_THREADS = 256;

// The semi-implicit update in the order of integrator.py:264-315.  Three
// places subtract nearly equal quantities, and the FP32 mode carries them in
// float-float (XF) so that the difference keeps FP32 relative precision:
// the divergence right-hand side (explicit tendency against the Laplacian of
// the geopotential), the temperature update (heating against the
// reference-temperature matrix on the mean divergence) and the pi update
// (against the column-integrated divergence).  WW and tmtx enter through
// their level-scan forms
//   (WW x)_k   = R alpha_k x_k + sum_{l<k} R dlog3_l x_l,
//   (tmtx D)_k = kappa Tref_k (alpha_k D_k + w3_k sum_{l>k} dsig_l D_l),
// each level summing its own prefix / suffix.  Damping factors 1 / (1 + c)
// are applied as x - x c / (1 + c) so that a small c keeps its precision.
template <typename R>
__global__ void __launch_bounds__(IM_THREADS) k_implicit(SD<R> d, R dt, int set, int ra_mode) {
  const int p = blockIdx.x, e = blockIdx.y;
  const int K = d.K, N = d.N, NS = d.NS;
  const int n1 = p, n2 = N - p;
  const int C1 = n1 + 1, C2n = (n2 != n1) ? n2 + 1 : 0;
  const int ncoef = C1 + C2n;
  const int CC = IM_THREADS / K;               // coefficients per chunk
  extern __shared__ unsigned char smraw[];
  R* mi = reinterpret_cast<R*>(smraw);          // [2][K][K] minv^T (l, k)
  R* vdT = mi + 2 * K * K;                      // [4][K][K] (vdiff - I)^T (l, k)
  R* vs = vdT + 4 * K * K;                      // [6][K] RALPHA RDLOG3 GG DSIG ALPHA W3
  R* ktr = vs + 6 * K;                          // [K] KTREF
  C2<R>* bA = reinterpret_cast<C2<R>*>(ktr + K + (K & 1));  // [CC][K]
  C2<R>* bB = bA + CC * K;                                   // [CC][K]
  const int tid = threadIdx.x;
  const R* mset = d.minv + (size_t)set * d.M * K * K;
  for (int idx = tid; idx < K * K; idx += IM_THREADS) {
    mi[idx] = mset[(size_t)n1 * K * K + idx];
    mi[K * K + idx] = mset[(size_t)n2 * K * K + idx];
  }
  for (int f = 0; f < 4; ++f)
    if (d.vd_on[f])
      for (int idx = tid; idx < K * K; idx += IM_THREADS)
        vdT[f * K * K + idx] = d.vdiff[((size_t)set * 4 + f) * K * K + idx];
  for (int idx = tid; idx < K; idx += IM_THREADS) {
    vs[0 * K + idx] = vrow(d, LBM_VERT_RALPHA, idx);
    vs[1 * K + idx] = vrow(d, LBM_VERT_RDLOG3, idx);
    vs[2 * K + idx] = vrow(d, LBM_VERT_GG, idx);
    vs[3 * K + idx] = vrow(d, LBM_VERT_DSIG, idx);
    vs[4 * K + idx] = vrow(d, LBM_VERT_ALPHA, idx);
    vs[5 * K + idx] = vrow(d, LBM_VERT_W3, idx);
    ktr[idx] = vrow(d, LBM_VERT_KTREF, idx);
  }
  __syncthreads();
  const R dt2 = R(2) * dt, gam = d.robert;
  const C2<R> z = cmk<R>(0, 0);
  const size_t e3 = (size_t)e * 4 * NS * K;
  const size_t efrc3 = d.frc_shared ? 0 : e3;
  const size_t efrcs = d.frc_shared ? 0 : (size_t)e * NS;
  for (int c0 = 0; c0 < ncoef; c0 += CC) {
    const int c = tid / K, k = tid % K;
    const int coef = c0 + c;
    const bool act = (c < CC) && (coef < ncoef);
    int n = 0, m = 0, sel = 0;
    if (act) {
      if (coef < C1) { n = n1; m = coef; sel = 0; }
      else { n = n2; m = coef - C1; sel = 1; }
    }
    const size_t idx = (size_t)spec_index(m, n, N);
    const size_t o = idx * K + k;
    C2<R> aV = z, aD = z, aT = z, aQ = z, bV = z, bD = z, bT = z, bQ = z;
    C2<R> wV = z, wD = z, wT = z, wQ = z, wpi = z, pp = z;
    R ktt = 0, kd = 0, kv = 0, kq = 0, lap = 0;
    if (act) {
      aV = d.sa3[e3 + 0 * NS * K + o]; aD = d.sa3[e3 + 1 * NS * K + o];
      aT = d.sa3[e3 + 2 * NS * K + o]; aQ = d.sa3[e3 + 3 * NS * K + o];
      bV = d.sb3[e3 + 0 * NS * K + o]; bD = d.sb3[e3 + 1 * NS * K + o];
      bT = d.sb3[e3 + 2 * NS * K + o]; bQ = d.sb3[e3 + 3 * NS * K + o];
      wV = d.tend[e3 + 0 * NS * K + o]; wD = d.tend[e3 + 1 * NS * K + o];
      wT = d.tend[e3 + 2 * NS * K + o]; wQ = d.tend[e3 + 3 * NS * K + o];
      wpi = d.tends[((size_t)e * 2 + 0) * NS + idx];
      pp = d.tends[((size_t)e * 2 + 1) * NS + idx];
      if (d.frc3) {
        wV = wV + d.frc3[efrc3 + 0 * NS * K + o]; wD = wD + d.frc3[efrc3 + 1 * NS * K + o];
        wT = wT + d.frc3[efrc3 + 2 * NS * K + o]; wQ = wQ + d.frc3[efrc3 + 3 * NS * K + o];
      }
      if (d.frcs) wpi = wpi + d.frcs[efrcs + idx];
      ktt = d.ktt[n * K + k]; kd = d.kd[n * K + k]; kv = d.kv[n * K + k]; kq = d.kq[n * K + k];
      lap = d.lap[n];
    }
    C2<R>* A = bA + c * K;
    C2<R>* B = bB + c * K;
    const R bt = dt2 * ktt;                      // 2 dt ktt; ft = 1 + bt
    __syncthreads();
    // wdx = T(t-dt) (1 + dt ktt) + dt wT  (integrator.py:287)
    if (act) A[k] = bT + (bT * ktt + wT) * dt;
    __syncthreads();
    if (act) {
      C2<R> pre = z;                                       // sum_{l<k} R dlog3_l wdx_l
      for (int l = 0; l < k; ++l) cfma(pre, vs[1 * K + l], A[l]);
      CX<R> phi = cx_add(cx_prod(vs[0 * K + k], A[k]), cx(pre));   // WW wdx
      const C2<R> wdpix = pp + wpi * dt;
      const R gk = vs[2 * K + k];
      // wdphiy = WW wdx + ft gg wdpix, ft gg taken as gg + bt gg
      phi = cx_add(phi, cx_add(cx_prod(gk, wdpix), cx_mul(cx_prod(bt, wdpix), gk)));
      // dt (wD ft - lap wdphiy), the two terms nearly balancing
      const CX<R> zz = cx_add(cx_add(cx(wD), cx_prod(bt, wD)), cx_mul(phi, -lap));
      const R ad = dt * kd;
      B[k] = bD + (bD * (ad + bt + ad * bt) + cx_val(zz) * dt);
    }
    __syncthreads();
    C2<R> dbar = z;
    if (act) {
      const R* mm_ = mi + sel * K * K;
      // M(n)^-1 rhs with exact products and compensated sums (the divergence
      // of a balanced flow is small against the terms of this sum)
      CX<R> acc = cx<R>(z);
      for (int l = 0; l < K; ++l) acc = cx_add(acc, cx_prod(mm_[l * K + k], B[l]));   // minv (l, k)
      dbar = cx_val(acc);
    }
    __syncthreads();
    if (act) A[k] = dbar;
    __syncthreads();
    C2<R> nV = z, nD = z, nT = z, nQ = z, npi = z;
    if (act) {
      C2<R> suf = z;                                        // sum_{l>k} dsig_l dbar_l
      for (int l = K - 1; l > k; --l) cfma(suf, vs[3 * K + l], A[l]);
      const CX<R> sfx = cx(suf);
      const CX<R> corr = cx_mul(cx_add(cx_prod(vs[4 * K + k], dbar), cx_mul(sfx, vs[5 * K + k])),
                                ktr[k]);
      const C2<R> yT = bT + cx_val(cx_add(cx(wT), cx_neg(corr))) * dt2;
      nT = yT - yT * (bt / (R(1) + bt));
      if (k == 0) {
        const CX<R> dsum = cx_add(sfx, cx_prod(vs[3 * K], dbar));
        npi = pp + cx_val(cx_add(cx(wpi), cx_neg(dsum))) * dt2;
      }
      nD = dbar * R(2) - bD;
      const R av = dt2 * kv, aq = dt2 * kq;
      const C2<R> xV = bV + wV * dt2, xQ = bQ + wQ * dt2;
      nV = xV - xV * (av / (R(1) + av));
      nQ = xQ - xQ * (aq / (R(1) + aq));
    }
    // implicit vertical diffusion (integrator.py:311-314); vdT holds the
    // operator minus the identity
    C2<R>* vals[4] = {&nV, &nD, &nT, &nQ};
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      if (!d.vd_on[f]) continue;
      __syncthreads();
      if (act) A[k] = *vals[f];
      __syncthreads();
      if (act && !(f < 2 && n < 2)) {
        C2<R> o2 = *vals[f];
        const R* vm = vdT + f * K * K;
        for (int l = 0; l < K; ++l) cfma(o2, vm[l * K + k], A[l]);
        *vals[f] = o2;
      }
    }
    // Robert-Asselin filter of the previous level (spectral part) and update
    if (act) {
      C2<R> fV, fD, fT, fQ;
      if (ra_mode) {
        fV = aV + (bV - aV * R(2) + nV) * gam;
        fD = aD + (bD - aD * R(2) + nD) * gam;
        fT = aT + (bT - aT * R(2) + nT) * gam;
        fQ = aQ + (bQ - aQ * R(2) + nQ) * gam;
      } else {
        fV = aV; fD = aD; fT = aT; fQ = aQ;
      }
      d.sb3[e3 + 0 * NS * K + o] = fV; d.sb3[e3 + 1 * NS * K + o] = fD;
      d.sb3[e3 + 2 * NS * K + o] = fT; d.sb3[e3 + 3 * NS * K + o] = fQ;
      d.sa3[e3 + 0 * NS * K + o] = nV; d.sa3[e3 + 1 * NS * K + o] = nD;
      d.sa3[e3 + 2 * NS * K + o] = nT; d.sa3[e3 + 3 * NS * K + o] = nQ;
      const bool fin = isfinite(nV.x) && isfinite(nV.y) && isfinite(nD.x) && isfinite(nD.y) &&
                       isfinite(nT.x) && isfinite(nT.y) && isfinite(nQ.x) && isfinite(nQ.y) &&
                       isfinite(npi.x) && isfinite(npi.y);
      if (!fin) {
        atomicOr(d.err, 1);
        if (d.err_member) atomicOr(d.err_member + e, 1);
      }
    }
    // column sums for sigma-dot of the next step
    __syncthreads();
    if (act) { A[k] = nV; B[k] = nD; }
    __syncthreads();
    if (act && k == 0) {
      C2<R> sv = z, sdv = z;
      for (int l = 0; l < K; ++l) {
        cfma(sv, vs[3 * K + l], A[l]);
        cfma(sdv, vs[3 * K + l], B[l]);
      }
      const R il = d.invlap[n];
      const size_t es = (size_t)e * 4 * NS;
      d.sas[es + 0 * NS + idx] = npi;
      d.sas[es + 1 * NS + idx] = sv * il;     // sum dsig psi
      d.sas[es + 2 * NS + idx] = sdv * il;    // sum dsig chi
      d.sas[es + 3 * NS + idx] = sdv;         // sum dsig div
    }
  }
}

// column sums of a freshly loaded current level
template <typename R>
__global__ void k_colsum(SD<R> d) {
  const int e = blockIdx.y;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int NS = d.NS, K = d.K;
  if (idx >= NS) return;
  int m = 0;
  while (m < d.N && spec_offset(m + 1, d.N) <= idx) ++m;
  const int n = m + (idx - spec_offset(m, d.N));
  const size_t e3 = (size_t)e * 4 * NS * K;
  C2<R> sv = cmk<R>(0, 0), sdv = cmk<R>(0, 0);
  for (int l = 0; l < K; ++l) {
    cfma(sv, vrow(d, LBM_VERT_DSIG, l), d.sa3[e3 + 0 * NS * K + (size_t)idx * K + l]);
    cfma(sdv, vrow(d, LBM_VERT_DSIG, l), d.sa3[e3 + 1 * NS * K + (size_t)idx * K + l]);
  }
  const R il = d.invlap[n];
  const size_t es = (size_t)e * 4 * NS;
  d.sas[es + 1 * NS + idx] = sv * il;
  d.sas[es + 2 * NS + idx] = sdv * il;
  d.sas[es + 3 * NS + idx] = sdv;
}

// Two adjacent complex values in one store (16 bytes in FP32; the six-field
// rows of sf start on 16-byte boundaries).
LBM_D void store_pair(C2<float>* o, C2<float> a, C2<float> b) {
  *reinterpret_cast<float4*>(o) = make_float4(a.x, a.y, b.x, b.y);
}
LBM_D void store_pair(C2<double>* o, C2<double> a, C2<double> b) {
  o[0] = a;
  o[1] = b;
}

// =============================================================================
// Legendre synthesis: state A -> sf, sfs, per (member, m-pair, level chunk)
// =============================================================================
constexpr int SY_THREADS = 320;

// SURF: only the surface fields (sfs), for the tensor-core synthesis, which
// computes the level fields (k_synth_tc).
template <typename R, int JG, int KC, int HV, bool SURF = false>
__global__ void __launch_bounds__(SY_THREADS, 2) k_synth(SD<R> d) {
  const int p = blockIdx.x, e = blockIdx.y, kc = blockIdx.z;
  const int J = d.J, K = d.K, N = d.N, M = d.M, JH = J / 2, NS = d.NS;
  const int k0 = kc * KC, kn = min(KC, K - k0);
  const PairRows<R> pr(p, N);
  extern __shared__ unsigned char smraw[];
  R* tp = reinterpret_cast<R*>(smraw);                 // [NR][JH]
  R* th = tp + pr.NR * JH;
  C2<R>* sv = reinterpret_cast<C2<R>*>(th + pr.NR * JH);    // [NR][6][KC]
  const int tid = threadIdx.x, nt = blockDim.x;
  const int off1 = spec_offset(pr.m1, N), off2 = spec_offset(pr.m2, N);
  for (int idx = tid; idx < pr.NR * JH; idx += nt) {
    const int r = idx / JH, jh = idx % JH;
    const int row = r < pr.L1 ? off1 + r : off2 + (r - pr.L1);
    tp[idx] = d.symp[(size_t)row * JH + jh];
    th[idx] = d.symh[(size_t)row * JH + jh];
  }
  const int nm = pr.L2 ? 2 : 1;
  if constexpr (!SURF) {
  const size_t e3 = (size_t)e * 4 * NS * K;
  for (int idx = tid; idx < pr.NR * kn; idx += nt) {
    const int r = idx / kn, kk = idx % kn;
    const int n = pr.n_of(r);
    const int row = r < pr.L1 ? off1 + r : off2 + (r - pr.L1);
    const size_t o = (size_t)row * K + k0 + kk;
    const C2<R> vo = d.sa3[e3 + 0 * (size_t)NS * K + o], dv = d.sa3[e3 + 1 * (size_t)NS * K + o];
    const R il = d.invlap[n];
    C2<R>* s = sv + (size_t)r * 6 * KC + kk;         // field f at s[f * KC]
    s[0 * KC] = vo * il;                               // psi
    s[1 * KC] = dv * il;                               // chi
    s[2 * KC] = vo;
    s[3 * KC] = dv;
    s[4 * KC] = d.sa3[e3 + 2 * (size_t)NS * K + o];
    s[5 * KC] = d.sa3[e3 + 3 * (size_t)NS * K + o];
  }
  __syncthreads();
  const int NJG = (JH + JG - 1) / JG;
  const size_t jmK = (size_t)J * K;
  C2<R>* sfe = d.sf + (size_t)e * M * jmK * SF_N;
  // Items: (term half, latitude group, level), level fastest.  With HV = 2
  // the first NJG KC items take the wind terms (P chi, H psi, P psi, H chi ->
  // U, V), the rest the scalar terms (P vor, P div, P T, P q): each value read
  // from shared memory then feeds JG latitudes of four terms, and the halves
  // are whole warps apart.  HV = 1: every item takes all eight terms.  Every
  // item walks the N + 2 rows of both m of the pair, so the pair's rows are
  // balanced across threads.
  const int nhalf = NJG * KC;
  for (int it = tid; it < HV * nhalf; it += nt) {
    const int half = HV == 2 ? (it >= nhalf ? 1 : 0) : -1;
    const int ri = it - (half > 0 ? nhalf : 0);
    const int kk = ri % KC;
    const int jg = ri / KC;
    if (kk >= kn) continue;
   for (int mm = 0; mm < nm; ++mm) {
    const int m = mm ? pr.m2 : pr.m1;
    const int rb = mm ? pr.L1 : 0, re = mm ? pr.NR : pr.L1;
    const R rm = R(m);
    // rows alternate parity of (n - m), starting even; P of an even row is
    // symmetric about the equator (plus), H of an even row antisymmetric.
    // acc[jg][term][plus/minus]
    auto wind = [&]() {
      C2<R> acc[JG][4][2];
#pragma unroll
      for (int a = 0; a < JG; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = cmk<R>(0, 0);
      auto row = [&](int r, auto par_tag) {
        constexpr int PP = decltype(par_tag)::value, HP = PP ^ 1;
        const C2<R>* sr = sv + r * 6 * KC + kk;
        const C2<R> psi = sr[0 * KC], chi = sr[1 * KC];
#pragma unroll
        for (int a = 0; a < JG; ++a) {
          const int jh = min(jg * JG + a, JH - 1);
          const R P = tp[r * JH + jh], H = th[r * JH + jh];
          cfma(acc[a][0][PP], P, chi);
          cfma(acc[a][1][HP], H, psi);
          cfma(acc[a][2][PP], P, psi);
          cfma(acc[a][3][HP], H, chi);
        }
      };
      for (int r = rb; r < re; r += 2) {
        row(r, std::integral_constant<int, 0>{});
        if (r + 1 < re) row(r + 1, std::integral_constant<int, 1>{});
      }
#pragma unroll
      for (int a = 0; a < JG; ++a) {
        const int jh = jg * JG + a;
        if (jh >= JH) break;
#pragma unroll
        for (int hemi = 0; hemi < 2; ++hemi) {
          const int j = hemi ? J - 1 - jh : jh;
          const R sg = hemi ? R(-1) : R(1);
          auto comb = [&](int b) { return acc[a][b][0] + acc[a][b][1] * sg; };
          C2<R>* o = sfe + (((size_t)m * J + j) * K + k0 + kk) * SF_N;
          store_pair(o + SF_U, im_mul(comb(0), rm) - comb(1), im_mul(comb(2), rm) + comb(3));
        }
      }
    };
    auto scalars = [&]() {
      C2<R> acc[JG][4][2];
#pragma unroll
      for (int a = 0; a < JG; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = cmk<R>(0, 0);
      auto row = [&](int r, auto par_tag) {
        constexpr int PP = decltype(par_tag)::value;
        const C2<R>* sr = sv + r * 6 * KC + kk;
        const C2<R> vo = sr[2 * KC], dv = sr[3 * KC], tt = sr[4 * KC], qq = sr[5 * KC];
#pragma unroll
        for (int a = 0; a < JG; ++a) {
          const int jh = min(jg * JG + a, JH - 1);
          const R P = tp[r * JH + jh];
          cfma(acc[a][0][PP], P, vo);
          cfma(acc[a][1][PP], P, dv);
          cfma(acc[a][2][PP], P, tt);
          cfma(acc[a][3][PP], P, qq);
        }
      };
      for (int r = rb; r < re; r += 2) {
        row(r, std::integral_constant<int, 0>{});
        if (r + 1 < re) row(r + 1, std::integral_constant<int, 1>{});
      }
#pragma unroll
      for (int a = 0; a < JG; ++a) {
        const int jh = jg * JG + a;
        if (jh >= JH) break;
#pragma unroll
        for (int hemi = 0; hemi < 2; ++hemi) {
          const int j = hemi ? J - 1 - jh : jh;
          const R sg = hemi ? R(-1) : R(1);
          auto comb = [&](int b) { return acc[a][b][0] + acc[a][b][1] * sg; };
          C2<R>* o = sfe + (((size_t)m * J + j) * K + k0 + kk) * SF_N;
          store_pair(o + SF_VOR, comb(0), comb(1));
          store_pair(o + SF_T, comb(2), comb(3));
        }
      }
    };
    if (half <= 0) wind();
    if (half != 0) scalars();
   }
  }
  }  // !SURF
  // surface fields (first level chunk only; the surface-only form takes
  // SURF_EB members per block)
  if constexpr (SURF) __syncthreads();
  auto surface = [&](int e) {
  const size_t es = (size_t)e * 4 * NS;
  for (int it = tid; it < nm * JH; it += nt) {
    const int jh = it % JH, mm = it / JH;
    const int m = mm ? pr.m2 : pr.m1;
    const int rb = mm ? pr.L1 : 0, re = mm ? pr.NR : pr.L1;
    const int offm = mm ? off2 : off1;
    // terms: Ppi Hpi Pchis Hpsis Ppsis Hchis Pds  [plus/minus]
    C2<R> acc[7][2];
#pragma unroll
    for (int b = 0; b < 7; ++b) acc[b][0] = acc[b][1] = cmk<R>(0, 0);
    auto row = [&](int r, auto par_tag) {
      constexpr int PP = decltype(par_tag)::value, HP = PP ^ 1;
      const size_t rowi = (size_t)offm + (r - rb);
      const C2<R> pi = d.sas[es + 0 * NS + rowi], psis = d.sas[es + 1 * NS + rowi];
      const C2<R> chis = d.sas[es + 2 * NS + rowi], ds = d.sas[es + 3 * NS + rowi];
      const R P = tp[r * JH + jh], H = th[r * JH + jh];
      cfma(acc[0][PP], P, pi);
      cfma(acc[1][HP], H, pi);
      cfma(acc[2][PP], P, chis);
      cfma(acc[3][HP], H, psis);
      cfma(acc[4][PP], P, psis);
      cfma(acc[5][HP], H, chis);
      cfma(acc[6][PP], P, ds);
    };
    for (int r = rb; r < re; r += 2) {
      row(r, std::integral_constant<int, 0>{});
      if (r + 1 < re) row(r + 1, std::integral_constant<int, 1>{});
    }
    const R rm = R(m);
    for (int hemi = 0; hemi < 2; ++hemi) {
      const int j = hemi ? J - 1 - jh : jh;
      const R sg = hemi ? R(-1) : R(1);
      auto comb = [&](int b) { return acc[b][0] + acc[b][1] * sg; };
      C2<R>* o = d.sfs + (((size_t)e * M + m) * J + j) * SFS_N;
      o[SFS_PI] = comb(0);
      o[SFS_PIY] = comb(1);
      o[SFS_UH] = im_mul(comb(2), rm) - comb(3);
      o[SFS_VH] = im_mul(comb(4), rm) + comb(5);
      o[SFS_DH] = comb(6);
    }
  }
  };
  if constexpr (SURF) {
    const int e1 = min(d.E, (int)(blockIdx.y + 1) * SURF_EB);
    for (int ee = blockIdx.y * SURF_EB; ee < e1; ++ee) surface(ee);
  } else {
    if (kc != 0) return;
    surface(e);
  }
}

// Apply the pending grid-ps update at the end of a run (see k_grid).
template <typename R, int I>
__global__ void k_ps_flush(SD<R> d, int ps_mode) {
  constexpr int R1 = FftShape<I>::R1;
  constexpr int SCR = fft_team_scratch<I>();
  const int j = blockIdx.x, e = blockIdx.y, J = d.J, M = d.M;
  __shared__ C2<R> tw[I];
  __shared__ C2<R> scr[SCR];
  __shared__ C2<R> X[I / 2];
  __shared__ R pi[I];
  const int tid = threadIdx.x;
  for (int p = tid; p < I; p += R1) tw[p] = d.tw[p];
  for (int m = tid; m < M; m += R1) X[m] = d.sfs[(((size_t)e * M + m) * J + j) * SFS_N + SFS_PI];
  __syncwarp();
  team_rfft_inv<I>(tid, [&](int m) { return X[m]; }, M, scr, tw, pi, 1, R(1));
  __syncwarp();
  for (int c = tid; c < I; c += R1) {
    const size_t g2 = (size_t)j * I + c;
    const size_t gp = (size_t)e * J * I + g2;
    const R psbar = d.b2[(B2_PSBAR * J) * I + g2];
    const R pscur = psbar * expm1(pi[c]);
    if (ps_mode == 1) {
      d.psb[gp] = d.psa[gp];
    } else if (ps_mode == 2) {
      const R pa = d.psa[gp];
      d.psb[gp] = pa + d.robert * (d.psb[gp] - R(2) * pa + pscur);
    }
    d.psa[gp] = pscur;
  }
}

}  // namespace lbm
#include "grid_split.cuh"
#include "legendre_tc.cuh"
#include "synth_tc.cuh"
#include "dft_tc.cuh"
namespace lbm {

// ---- launch configuration ------------------------------------------------------
template <typename R> struct Cfg;
template <> struct Cfg<float> {
  static constexpr int NC = 4, KCA = 20, JG = 4, KCS = 20, SHV = 2;
};
template <> struct Cfg<double> {
  static constexpr int NC = 2, KCA = 10, JG = 1, KCS = 10, SHV = 1;
};

template <typename R, int I> constexpr int grid_kb() { return (sizeof(R) == 8 && I == 256) ? 2 : 4; }
template <typename R, int I> constexpr int grid_nt() {
  return I == 64 ? 128 : ((I == 256 && sizeof(R) == 8) ? 128 : 256);
}

template <typename R> size_t anal_smem(int N, int JH, int KC) {
  constexpr int NC = Cfg<R>::NC;
  const size_t TS = (size_t)NC * anal_groups<NC>(N) + 1;
  return sizeof(R) * 2 * TS * JH + 16 + sizeof(C2<R>) * (size_t)2 * (2 * AN_JC * 2 * AF_N * KC);
}
// Level chunk of the analysis block (one thread per level and row group): the
// preferred Cfg<R>::KCA, halved where that block would exceed 256 threads.
template <typename R> int anal_kc(int N) {
  constexpr int NC = Cfg<R>::NC;
  const int G = anal_groups<NC>(N);
  return (Cfg<R>::KCA * G > 256) ? Cfg<R>::KCA / 2 : Cfg<R>::KCA;
}
template <typename R, int KC> void launch_anal(const SD<R>& d, cudaStream_t st, bool attrs) {
  constexpr int NC = Cfg<R>::NC;
  const int JH = d.J / 2, NRmax = d.N + 2, NP = (d.M + 1) / 2;
  const int G = anal_groups<NC>(d.N);
  const int nt = ((KC * G + 31) / 32) * 32;
  // the surface pass also needs 2 * JH * 2 staging elements
  size_t sm = anal_smem<R>(d.N, JH, KC);
  const size_t sm2 = sizeof(R) * 2 * ((size_t)NC * G + 1) * JH + 16 +
                     sizeof(C2<R>) * (size_t)2 * JH * 2 * 2;
  if (sm2 > sm) sm = sm2;
  if (attrs) {
    cudaFuncSetAttribute(k_anal<R, NC, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(k_anal<R, NC, KC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
  } else if (d.legendre && !(d.tc_off & 1) && sizeof(R) == 4) {
    k_anal<R, NC, KC, true><<<dim3(NP, (d.E + SURF_EB - 1) / SURF_EB, 1), nt, sm, st>>>(d);
  } else {
    k_anal<R, NC, KC><<<dim3(NP, d.E, (d.K + KC - 1) / KC), nt, sm, st>>>(d);
  }
}
template <typename R> void run_anal(const SD<R>& d, cudaStream_t st, bool attrs) {
  if (anal_kc<R>(d.N) == Cfg<R>::KCA) launch_anal<R, Cfg<R>::KCA>(d, st, attrs);
  else launch_anal<R, Cfg<R>::KCA / 2>(d, st, attrs);
}
inline int persistent_grid(const void* fn, int nt, size_t smem, int units);
template <typename R> size_t synth_smem(int NR, int JH) {
  return sizeof(R) * 2 * (size_t)NR * JH + sizeof(C2<R>) * (size_t)NR * Cfg<R>::KCS * 6;
}
// Legendre synthesis launch: HV NJG KC items, at most SY_THREADS threads.
template <typename R> void launch_synth(const SD<R>& d, cudaStream_t st) {
  constexpr int JG = Cfg<R>::JG, KC = Cfg<R>::KCS, HV = Cfg<R>::SHV;
  const int JH = d.J / 2, NRmax = d.N + 2, NP = (d.M + 1) / 2;
  const int NJG = (JH + JG - 1) / JG;
  int nt = HV * NJG * KC;
  nt = nt > SY_THREADS ? SY_THREADS : ((nt + 31) / 32) * 32;
  if constexpr (sizeof(R) == 4) {
    if (d.legendre && !(d.tc_off & 2)) {
      // level fields on the tensor cores, surface fields by the FMA kernel
      const StcPlan pl = stc_plan(d.E, d.J, d.K, d.N, d.tc_g);
      k_synth_tc<<<persistent_grid((const void*)k_synth_tc, STC_THREADS, pl.smem, pl.nunits),
                   STC_THREADS, pl.smem, st>>>(d, d.tc_synth, pl, d.legendre);
      k_synth<R, JG, KC, HV, true><<<dim3(NP, (d.E + SURF_EB - 1) / SURF_EB, 1), nt,
                                       synth_smem<R>(NRmax, JH), st>>>(d);
      return;
    }
  }
  k_synth<R, JG, KC, HV><<<dim3(NP, d.E, (d.K + KC - 1) / KC), nt, synth_smem<R>(NRmax, JH),
                           st>>>(d);
}
template <typename R> size_t impl_smem(int K) {
  return sizeof(R) * ((size_t)(2 + 4) * K * K + 7 * (size_t)K + (K & 1)) +
         sizeof(C2<R>) * 2 * (size_t)(IM_THREADS / K) * K;
}

// Grid of a persistent kernel: the CTAs that are resident at once on the
// current device (from the occupancy calculator, cached per kernel, block
// size, shared memory and device), at most `units`.
inline int persistent_grid(const void* fn, int nt, size_t smem, int units) {
  struct Entry { const void* fn; int nt, dev; size_t smem; int ctas; };
  static std::mutex mu;
  static Entry cache[32];
  static int ncache = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  int ctas = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < ncache; ++i)
      if (cache[i].fn == fn && cache[i].nt == nt && cache[i].dev == dev && cache[i].smem == smem)
        ctas = cache[i].ctas;
    if (!ctas) {
      int sms = 0, per = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, nt, smem);
      ctas = (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
      if (ncache < 32) cache[ncache++] = Entry{fn, nt, dev, smem, ctas};
    }
  }
  return ctas < units ? ctas : units;
}

template <typename R, int I> int launch_step(const SD<R>& d, const lbm_step_ctl& c,
                                             cudaStream_t st, int only = -1) {
  constexpr int KB = grid_kb<R, I>(), NT = grid_nt<R, I>();
  const int NP = (d.M + 1) / 2;
  const int JH = d.J / 2;
  const int NRmax = d.N + 2;
  const size_t gsm = GridSmem<R, I, KB, NT>::bytes(d.M);
  if constexpr (sizeof(R) == 4) {
    // grid-point part as three launches: longitude synthesis, column
    // algebra, longitude analysis (kernel ids 4, 5, 6; 0 = all three)
    if (only < 0 || only == 0 || only == 4)
      k_idft<I><<<dim3(d.J, d.E), IDFT_NT, idft_smem(I, d.M), st>>>(d, d.dft);
    if (only < 0 || only == 0 || only == 5)
      k_alg<I><<<dim3(d.J, d.E), I, 0, st>>>(d, c.ps_mode);
    if ((only < 0 || only == 0 || only == 6) && d.legendre && !(d.tc_off & 4) &&
        ftc_supported(I, d.K, d.N)) {
      const FtcPlan pl = ftc_plan(d.E, d.J, I, d.K, d.N);
      k_fdft_tc<<<persistent_grid((const void*)k_fdft_tc, FTC_THREADS, pl.smem, pl.nunits),
                  FTC_THREADS, pl.smem, st>>>(d, d.tc_dft, pl, d.legendre);
      // the surface rows on the FMA pipes; their FP32 cos table follows the
      // tensor-core image
      k_fdft_surf<<<dim3(d.J, (d.E + FSURF_EB - 1) / FSURF_EB), 128, fsurf_smem(I), st>>>(
          d, reinterpret_cast<const float*>(d.tc_dft + pl.tab_bytes));
    } else if (only < 0 || only == 0 || only == 6) {
      const FdftPlan pl = fdft_plan(I, d.M, d.K);
      const size_t smem = sizeof(float) * (size_t)pl.total;
      const int nunits = d.E * d.J * ((d.K + pl.lc - 1) / pl.lc);
      k_fdft<I><<<persistent_grid((const void*)k_fdft<I>, pl.nt, smem, nunits), pl.nt, smem,
                  st>>>(d, d.dft, pl);
    }
  } else {
    if (only < 0 || only == 0)
      k_grid<R, I, KB, NT><<<dim3(d.J, d.E), NT, gsm, st>>>(d, c.ps_mode);
  }
  if (only < 0 || only == 1) {
    if constexpr (sizeof(R) == 4) {
      if (d.legendre && !(d.tc_off & 1)) {
        const AtcPlan pl = atc_plan(d.E, d.J, d.K, d.N, d.tc_g);
        k_anal_tc<<<persistent_grid((const void*)k_anal_tc, ATC_THREADS, pl.smem, pl.nunits),
                    ATC_THREADS, pl.smem, st>>>(d, d.tc_anal, pl, d.legendre);
      }
    }
    run_anal<R>(d, st, false);
  }
  if (only < 0 || only == 2)
    k_implicit<R><<<dim3(NP, d.E), IM_THREADS, impl_smem<R>(d.K), st>>>(d, R(c.dt), c.set,
                                                                         c.ra_mode);
  if (only < 0 || only == 3) launch_synth<R>(d, st);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

template <typename R, int I> void set_attrs(const SD<R>& d) {
  constexpr int KB = grid_kb<R, I>(), NT = grid_nt<R, I>();
  const int JH = d.J / 2, NRmax = d.N + 2;
  if constexpr (sizeof(R) == 4) {
    cudaFuncSetAttribute(k_idft<I>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)idft_smem(I, d.M));
    const FdftPlan pl = fdft_plan(I, d.M, d.K);
    const size_t smem = sizeof(float) * (size_t)pl.total;
    if (smem <= 227 * 1024) {
      cudaFuncSetAttribute(k_fdft<I>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      persistent_grid((const void*)k_fdft<I>, pl.nt, smem, 1);
    }
    if (d.legendre && ftc_supported(I, d.K, d.N)) {
      const FtcPlan fp = ftc_plan(d.E, d.J, I, d.K, d.N);
      cudaFuncSetAttribute(k_fdft_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fp.smem);
      persistent_grid((const void*)k_fdft_tc, FTC_THREADS, fp.smem, 1);
    }
  } else {
    cudaFuncSetAttribute(k_grid<R, I, KB, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)GridSmem<R, I, KB, NT>::bytes(d.M));
  }
  run_anal<R>(d, nullptr, true);
  if constexpr (sizeof(R) == 4) {
    if (d.legendre) {
      const AtcPlan pl = atc_plan(d.E, d.J, d.K, d.N, d.tc_g);
      cudaFuncSetAttribute(k_anal_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
      persistent_grid((const void*)k_anal_tc, ATC_THREADS, pl.smem, 1);
    }
  }
  cudaFuncSetAttribute(k_implicit<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)impl_smem<R>(d.K));
  cudaFuncSetAttribute(k_synth<R, Cfg<R>::JG, Cfg<R>::KCS, Cfg<R>::SHV>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)synth_smem<R>(NRmax, JH));
  cudaFuncSetAttribute(k_synth<R, Cfg<R>::JG, Cfg<R>::KCS, Cfg<R>::SHV, true>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)synth_smem<R>(NRmax, JH));
  if constexpr (sizeof(R) == 4) {
    if (d.legendre) {
      const StcPlan pl = stc_plan(d.E, d.J, d.K, d.N, d.tc_g);
      cudaFuncSetAttribute(k_synth_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
      persistent_grid((const void*)k_synth_tc, STC_THREADS, pl.smem, 1);
    }
  }
}

template <typename R> int validate(const SD<R>& d) {
  if (d.E < 1 || d.K < 1 || d.K > 64 || d.N < 1 || (d.J & 1) || 2 * d.M > d.I) return LBM_ERR_ARG;
  if (d.I != 64 && d.I != 128 && d.I != 256) return LBM_ERR_ARG;
  if (IM_THREADS / d.K < 1) return LBM_ERR_ARG;
  if (!d.symp || !d.symh || !d.tw || !d.jfac || !d.vert || !d.b3 || !d.bsd || !d.b2 ||
      !d.lap || !d.invlap || !d.nn1a || !d.kv || !d.kd || !d.ktt || !d.kq ||
      !d.minv || !d.sa3 || !d.sas || !d.sb3 || !d.psa || !d.psb || !d.sf ||
      !d.sfs || !d.af || !d.afs || !d.tend || !d.tends || !d.err)
    return LBM_ERR_ARG;
  for (int f = 0; f < 4; ++f)
    if (d.vd_on[f] && !d.vdiff) return LBM_ERR_ARG;
  if (sizeof(R) == 4 && (!d.dft || !d.grid6 || !d.grid9)) return LBM_ERR_ARG;
  // 16-byte copies and bulk prefetches read sf, af and grid9
  auto a16 = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
  if (!a16(d.sf) || !a16(d.af) || (sizeof(R) == 4 && !a16(d.grid9))) return LBM_ERR_ARG;
  if (d.legendre) {
    // tensor-core analysis: FP32 state, 16-latitude steps, 16-byte af rows,
    // at most 256 table rows, the plan within shared memory
    if (sizeof(R) != 4 || (d.legendre != 3 && d.legendre != 6) || !d.tc_anal ||
        !d.tc_synth || (d.J % 16) || (d.K & 1) || d.M > 256 ||
        atc_plan(d.E, d.J, d.K, d.N, d.tc_g).smem > 227 * 1024 ||
        stc_plan(d.E, d.J, d.K, d.N, d.tc_g).smem > 227 * 1024 ||
        (stc_plan(d.E, d.J, d.K, d.N).JT % 16) || d.tc_off < 0 || d.tc_off > 7 ||
        d.tc_g < 0 ||
        (ftc_supported(d.I, d.K, d.N) &&
         (!d.tc_dft || ((uintptr_t)d.tc_dft & 15) ||
          ftc_plan(d.E, d.J, d.I, d.K, d.N).smem > 227 * 1024)) ||
        ((uintptr_t)d.tc_anal & 15) || ((uintptr_t)d.tc_synth & 15))
      return LBM_ERR_ARG;
  }
  if (sizeof(R) == 4 &&
      (idft_smem(d.I, d.M) > 227 * 1024 ||
       sizeof(float) * (size_t)fdft_plan(d.I, d.M, d.K).total > 227 * 1024))
    return LBM_ERR_ARG;
  return LBM_OK;
}

template <typename R> int run_steps(const lbm_stepper_desc* desc, const lbm_step_ctl* ctl,
                                    int nsteps, cudaStream_t st) {
  const SD<R> d = make_sd<R>(*desc);
  int rc = validate(d);
  if (rc) return rc;
  for (int s = 0; s < nsteps; ++s) {
    if (ctl[s].set < 0 || ctl[s].set >= d.nsets) return LBM_ERR_ARG;
    switch (d.I) {
      case 64: rc = launch_step<R, 64>(d, ctl[s], st); break;
      case 128: rc = launch_step<R, 128>(d, ctl[s], st); break;
      default: rc = launch_step<R, 256>(d, ctl[s], st); break;
    }
    if (rc) return rc;
  }
  return LBM_OK;
}

template <typename R> int launch_one(const lbm_stepper_desc* desc, const lbm_step_ctl& c,
                                     int kernel, cudaStream_t st) {
  const SD<R> d = make_sd<R>(*desc);
  int rc = validate(d);
  if (rc) return rc;
  if (c.set < 0 || c.set >= d.nsets) return LBM_ERR_ARG;
  switch (d.I) {
    case 64: return launch_step<R, 64>(d, c, st, kernel);
    case 128: return launch_step<R, 128>(d, c, st, kernel);
    default: return launch_step<R, 256>(d, c, st, kernel);
  }
}

template <typename R> int prepare_attrs(const lbm_stepper_desc* desc) {
  const SD<R> d = make_sd<R>(*desc);
  int rc = validate(d);
  if (rc) return rc;
  {
    // the analysis block holds one thread per (level, row group) of an m-pair
    constexpr int NC = Cfg<R>::NC;
    const int KC = anal_kc<R>(d.N);
    const int G = anal_groups<NC>(d.N);
    const int nt = ((KC * G + 31) / 32) * 32;
    cudaFuncAttributes fa;
    const cudaError_t ea = (KC == Cfg<R>::KCA)
                               ? cudaFuncGetAttributes(&fa, k_anal<R, NC, Cfg<R>::KCA>)
                               : cudaFuncGetAttributes(&fa, k_anal<R, NC, Cfg<R>::KCA / 2>);
    if (ea != cudaSuccess) return LBM_ERR_LAUNCH;
    if (nt > fa.maxThreadsPerBlock) return LBM_ERR_ARG;
  }
  switch (d.I) {
    case 64: set_attrs<R, 64>(d); break;
    case 128: set_attrs<R, 128>(d); break;
    default: set_attrs<R, 256>(d); break;
  }
  return cudaGetLastError() == cudaSuccess ? LBM_OK : LBM_ERR_LAUNCH;
}

template <typename R> int prime(const lbm_stepper_desc* desc, cudaStream_t st) {
  const SD<R> d = make_sd<R>(*desc);
  int rc = validate(d);
  if (rc) return rc;
  launch_synth<R>(d, st);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

template <typename R> int colsum(const lbm_stepper_desc* desc, cudaStream_t st) {
  const SD<R> d = make_sd<R>(*desc);
  int rc = validate(d);
  if (rc) return rc;
  k_colsum<R><<<dim3((d.NS + 127) / 128, d.E), 128, 0, st>>>(d);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

template <typename R> int flush(const lbm_stepper_desc* desc, int ps_mode, cudaStream_t st) {
  const SD<R> d = make_sd<R>(*desc);
  int rc = validate(d);
  if (rc) return rc;
  switch (d.I) {
    case 64: k_ps_flush<R, 64><<<dim3(d.J, d.E), FftShape<64>::R1, 0, st>>>(d, ps_mode); break;
    case 128: k_ps_flush<R, 128><<<dim3(d.J, d.E), FftShape<128>::R1, 0, st>>>(d, ps_mode); break;
    default: k_ps_flush<R, 256><<<dim3(d.J, d.E), FftShape<256>::R1, 0, st>>>(d, ps_mode); break;
  }
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

// ---- stepping from a static scratch area ------------------------------------
// lbm_stepper_run_noalloc takes the intermediate buffers of a step (sf, sfs,
// af, afs, tend, tends and in FP32 mode grid6, grid9) from this file-scope
// array instead of caller memory.  It is sized once, at LBM_NOALLOC_SCRATCH_BYTES, and every GPU that
// loads the library holds it until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[LBM_NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static void* g_noalloc_base[NOALLOC_MAX_DEVICES];

// Byte offsets of sf, sfs, af, afs, tend, tends (and in FP32 mode grid6,
// grid9) in the scratch area, each rounded up to 256 bytes.  `need` is the
// total, computed in double so that an absurd size cannot wrap around before
// it is compared with the maximum.
static void noalloc_layout(const lbm_stepper_desc& d, size_t off[8], double* need) {
  const double c = 2.0 * (d.prec == LBM_F64 ? sizeof(double) : sizeof(float));
  const double E = d.nmem, M = d.nmax + 1.0, J = d.nlat, K = d.kmax, I = d.nlon;
  const double NS = M * (M + 1.0) / 2.0;
  const double g = (d.prec == LBM_F32) ? 1.0 : 0.0;
  const double bytes[8] = {c * E * M * J * K * 6, c * E * M * J * 5, c * E * M * J * K * 7,
                           c * E * M * J * 2,     c * E * 4 * NS * K, c * E * 2 * NS,
                           g * 4.0 * E * J * (6 + 6 * K) * I, g * 4.0 * E * J * (2 + 9 * K) * I};
  double t = 0.0;
  for (int i = 0; i < 8; ++i) {
    off[i] = (size_t)t;
    t += 256.0 * std::ceil(bytes[i] / 256.0);
  }
  *need = t;
}

// Device address of the scratch area on the current device.  The first call
// on a device looks it up with cudaGetSymbolAddress (with that device
// current) and keeps it; later calls reuse it.  The address belongs to the
// device's primary context (the one the CUDA runtime uses): a caller running
// under another context of its own, or one that resets the device after the
// first call, would be handed an address that is no longer valid there.
static int noalloc_base(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return LBM_ERR_LAUNCH;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_base[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return LBM_ERR_LAUNCH;
    g_noalloc_base[dev] = p;
  }
  *out = g_noalloc_base[dev];
  return LBM_OK;
}

template <typename R> int run_noalloc(const lbm_stepper_desc& w, const lbm_step_ctl* ctl,
                                      int nsteps, size_t clear, cudaStream_t st) {
  // the full argument check runs before the clear, capturing or not
  const int vrc = validate(make_sd<R>(w));
  if (vrc) return vrc;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  if (cs == cudaStreamCaptureStatusNone) {
    const int rc = prepare_attrs<R>(&w);
    if (rc) return rc;
  }
  if (cudaMemsetAsync(w.sf, 0, clear, st) != cudaSuccess) return LBM_ERR_LAUNCH;
  const int rc = prime<R>(&w, st);
  if (rc) return rc;
  return run_steps<R>(&w, ctl, nsteps, st);
}

}  // namespace lbm

using namespace lbm;

struct lbm_graph {
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

extern "C" {

int lbm_stepper_prime(const lbm_stepper_desc* d, void* stream) {
  if (!d) return LBM_ERR_ARG;
  int rc = d->prec == LBM_F64 ? prepare_attrs<double>(d) : prepare_attrs<float>(d);
  if (rc) return rc;
  return d->prec == LBM_F64 ? prime<double>(d, (cudaStream_t)stream)
                            : prime<float>(d, (cudaStream_t)stream);
}

int lbm_stepper_run(const lbm_stepper_desc* d, const lbm_step_ctl* ctl, int nsteps,
                    void* stream) {
  if (!d || !ctl || nsteps < 0 || (d->prec != LBM_F64 && d->prec != LBM_F32)) return LBM_ERR_ARG;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing((cudaStream_t)stream, &cs);
  if (cs == cudaStreamCaptureStatusNone) {
    int rc = d->prec == LBM_F64 ? prepare_attrs<double>(d) : prepare_attrs<float>(d);
    if (rc) return rc;
  }
  return d->prec == LBM_F64 ? run_steps<double>(d, ctl, nsteps, (cudaStream_t)stream)
                            : run_steps<float>(d, ctl, nsteps, (cudaStream_t)stream);
}

int lbm_stepper_launch(const lbm_stepper_desc* d, const lbm_step_ctl* ctl, int kernel,
                       void* stream) {
  if (!d || !ctl || kernel < 0 || kernel > 6 || (d->prec != LBM_F64 && d->prec != LBM_F32) ||
      (kernel > 3 && d->prec != LBM_F32))
    return LBM_ERR_ARG;
  int rc = d->prec == LBM_F64 ? prepare_attrs<double>(d) : prepare_attrs<float>(d);
  if (rc) return rc;
  return d->prec == LBM_F64 ? launch_one<double>(d, *ctl, kernel, (cudaStream_t)stream)
                            : launch_one<float>(d, *ctl, kernel, (cudaStream_t)stream);
}

int lbm_stepper_flush(const lbm_stepper_desc* d, int ps_mode, void* stream) {
  if (!d || ps_mode < 0 || ps_mode > 2) return LBM_ERR_ARG;
  return d->prec == LBM_F64 ? flush<double>(d, ps_mode, (cudaStream_t)stream)
                            : flush<float>(d, ps_mode, (cudaStream_t)stream);
}

int lbm_stepper_colsum(const lbm_stepper_desc* d, void* stream) {
  if (!d) return LBM_ERR_ARG;
  return d->prec == LBM_F64 ? colsum<double>(d, (cudaStream_t)stream)
                            : colsum<float>(d, (cudaStream_t)stream);
}

int lbm_graph_capture(const lbm_stepper_desc* d, const lbm_step_ctl* ctl, int nsteps,
                      void* stream, lbm_graph** out) {
  if (!d || !ctl || !out || nsteps < 1) return LBM_ERR_ARG;
  int rc = d->prec == LBM_F64 ? prepare_attrs<double>(d) : prepare_attrs<float>(d);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return LBM_ERR_LAUNCH;
  rc = d->prec == LBM_F64 ? run_steps<double>(d, ctl, nsteps, st)
                          : run_steps<float>(d, ctl, nsteps, st);
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(st, &g);
  if (rc || ec != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    return rc ? rc : LBM_ERR_LAUNCH;
  }
  cudaGraphExec_t ex = nullptr;
  if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    return LBM_ERR_LAUNCH;
  }
  lbm_graph* h = new (std::nothrow) lbm_graph;
  if (!h) {
    cudaGraphExecDestroy(ex);
    cudaGraphDestroy(g);
    return LBM_ERR_LAUNCH;
  }
  h->graph = g;
  h->exec = ex;
  *out = h;
  return LBM_OK;
}

int lbm_graph_launch(lbm_graph* g, void* stream) {
  if (!g) return LBM_ERR_ARG;
  return cudaGraphLaunch(g->exec, (cudaStream_t)stream) == cudaSuccess ? LBM_OK
                                                                       : LBM_ERR_LAUNCH;
}

int lbm_graph_destroy(lbm_graph* g) {
  if (!g) return LBM_ERR_ARG;
  cudaGraphExecDestroy(g->exec);
  cudaGraphDestroy(g->graph);
  delete g;
  return LBM_OK;
}

int lbm_stepper_run_noalloc(const lbm_stepper_desc* d, const lbm_step_ctl* ctl, int nsteps,
                            void* stream) {
  if (!d || !ctl || nsteps < 0 || (d->prec != LBM_F64 && d->prec != LBM_F32)) return LBM_ERR_ARG;
  if (d->nmem < 1 || d->nlat < 2 || d->nmax < 1 || d->kmax < 1) return LBM_ERR_ARG;
  if (d->nlon != 64 && d->nlon != 128 && d->nlon != 256) return LBM_ERR_ARG;
  size_t off[8];
  double need = 0.0;
  noalloc_layout(*d, off, &need);
  if (!(need > 0.0)) return LBM_ERR_ARG;
  if (need > (double)LBM_NOALLOC_SCRATCH_BYTES) return LBM_ERR_SCRATCH;
  for (int s = 0; s < nsteps; ++s)
    if (ctl[s].set < 0 || ctl[s].set >= d->nsets || ctl[s].ps_mode < 0 || ctl[s].ps_mode > 2 ||
        ctl[s].ra_mode < 0 || ctl[s].ra_mode > 1)
      return LBM_ERR_ARG;
  void* base = nullptr;
  const int rc = noalloc_base(&base);
  if (rc) return rc;
  unsigned char* b = static_cast<unsigned char*>(base);
  lbm_stepper_desc w = *d;
  w.sf = b + off[0];
  w.sfs = b + off[1];
  w.af = b + off[2];
  w.afs = b + off[3];
  w.tend = b + off[4];
  w.tends = b + off[5];
  w.grid6 = d->prec == LBM_F32 ? b + off[6] : nullptr;
  w.grid9 = d->prec == LBM_F32 ? b + off[7] : nullptr;
  const size_t clear = (size_t)need;
  cudaStream_t st = (cudaStream_t)stream;
  return d->prec == LBM_F64 ? run_noalloc<double>(w, ctl, nsteps, clear, st)
                            : run_noalloc<float>(w, ctl, nsteps, clear, st);
}

}  // extern "C"
