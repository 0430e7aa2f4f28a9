// Adjoints of the two per-column / per-coefficient linear maps of the time
// step, written once for the device kernels (adjoint.cu) and for host
// compilation (the CPU tests build this header with g++ and check it
// against the forward formulas).  Plain real arithmetic, no CUDA types.
//
// Forward maps (reference dynamics.py:156-271 and integrator.py:264-315):
//  * grid-point tendency, one column: inputs u v t q vor div [K] and pi_x
//    pi_y; outputs fu fv ke gt xu xv g yu yv [K] and gt_pi.  Linear about
//    the basic state except the kinetic energy 0.5 (u^2 + v^2), which is
//    linearised about a trajectory (u0, v0): ke += u0 u + v0 v.
//  * semi-implicit leapfrog update, one (m, n) coefficient: linear in the
//    previous level and the explicit tendencies, real coefficients, so the
//    real and imaginary parts go through the same transpose.
#pragma once

#if defined(__CUDACC__)
#define LBM_COL_HD __host__ __device__ inline
#else
#define LBM_COL_HD inline
#endif

namespace lbm_adj {

// Transpose of the f-argument of the vertical advection operator
//   VA(f; s)[k] = (fhi - flo - f[k] (s[k+1] - s[k])) / dsig[k],
//   flo = s[k] (f[k] + f[k-1]) / 2 for k >= 1, fhi = s[k+1] (f[k+1] + f[k]) / 2
//   for k + 1 <= K - 1 (reference dynamics.py:117-143): fbar += dVA/df^T y.
template <typename R>
LBM_COL_HD void va_f_adj(int k, int K, R y, const R* s, const R* dsig, R* fbar) {
  const R z = y / dsig[k];
  if (k + 1 <= K - 1) {
    const R h = R(0.5) * s[k + 1] * z;
    fbar[k + 1] += h;
    fbar[k] += h;
  }
  if (k >= 1) {
    const R h = R(0.5) * s[k] * z;
    fbar[k] -= h;
    fbar[k - 1] -= h;
  }
  fbar[k] -= z * (s[k + 1] - s[k]);
}

// Transpose of the s-argument (s has K + 1 entries).
template <typename R>
LBM_COL_HD void va_s_adj(int k, int K, R y, const R* f, const R* dsig, R* sbar) {
  const R z = y / dsig[k];
  if (k + 1 <= K - 1) sbar[k + 1] += R(0.5) * (f[k + 1] + f[k]) * z;
  if (k >= 1) sbar[k] -= R(0.5) * (f[k] + f[k - 1]) * z;
  sbar[k + 1] -= z * f[k];
  sbar[k] += z * f[k];
}

// Vertical constants and one column of the basic state.
template <typename R>
struct ColConst {
  int K;
  R kappa, eps, rair;
  const R *dsig, *sigm, *alpha, *w3, *wP, *cpg, *ww, *tmtx, *tref;    // [K] / [K+1] / [K][K]
  const R *ub, *vb, *tb, *qb, *tvb, *absv, *divb, *x5b, *sdb;         // [K], sdb [K+1]
  R pixb, piyb;
  const R *u0, *v0;   // linearisation trajectory of the kinetic energy, or null
};

// Adjoint of the grid-point tendency of one column.  Inputs: adjoints of
// fu fv ke gt xu xv g yu yv (each [K]) and of gt_pi.  Outputs (overwritten):
// adjoints of u v t q vor div ([K]) and of pi_x, pi_y.  Scratch: 5 (K + 1)
// values in `work`.
template <typename R>
LBM_COL_HD void tendency_column_adjoint(const ColConst<R>& c, const R* afu, const R* afv,
                                        const R* ake, const R* agt, const R* axu,
                                        const R* axv, const R* ag, const R* ayu,
                                        const R* ayv, R agtpi, R* au, R* av, R* at, R* aq,
                                        R* avor, R* adiv, R* apix, R* apiy, R* work) {
  const int K = c.K;
  R* atv = work;                 // adjoint of tv' [K]
  R* ax5 = atv + (K + 1);        // adjoint of the omega factor x5' [K]
  R* apadv = ax5 + (K + 1);      // adjoint of v'.grad(ln ps) terms [K]
  R* aS = apadv + (K + 1);       // adjoint of the column sums S [K+1]
  R* asd = aS + (K + 1);         // adjoint of sigma-dot [K+1]
  for (int k = 0; k <= K; ++k) {
    atv[k] = ax5[k] = apadv[k] = aS[k] = asd[k] = R(0);
  }
  for (int k = 0; k < K; ++k) au[k] = av[k] = at[k] = aq[k] = avor[k] = adiv[k] = R(0);
  R px = R(0), py = R(0);
  for (int k = 0; k < K; ++k) {
    const R tdev = c.tb[k] - c.tref[k], tvdev = c.tvb[k] - c.tref[k];
    const R rcpg = c.rair * c.cpg[k];
    // gt = -kappa (tv' x5b + tvb x5') + t' divb + tdev div' + VA(t'; sdb)
    //      + VA(tb; sd') + sum_l tmtx[k][l] div'_l
    const R g = agt[k];
    atv[k] -= c.kappa * c.x5b[k] * g;
    ax5[k] -= c.kappa * c.tvb[k] * g;
    at[k] += c.divb[k] * g;
    adiv[k] += tdev * g;
    va_f_adj(k, K, g, c.sdb, c.dsig, at);
    va_s_adj(k, K, g, c.tb, c.dsig, asd);
    for (int l = 0; l < K; ++l) adiv[l] += c.tmtx[k * K + l] * g;
    // xu = u' tdev + ub t', xv = v' tdev + vb t'
    au[k] += tdev * axu[k];
    at[k] += c.ub[k] * axu[k];
    av[k] += tdev * axv[k];
    at[k] += c.vb[k] * axv[k];
    // fu = v' absv + vb vor' - rcpg (tv' pixb + tvdev pi_x) + VA(u'; sdb) + VA(ub; sd')
    R f = afu[k];
    av[k] += c.absv[k] * f;
    avor[k] += c.vb[k] * f;
    atv[k] -= rcpg * c.pixb * f;
    px -= rcpg * tvdev * f;
    va_f_adj(k, K, f, c.sdb, c.dsig, au);
    va_s_adj(k, K, f, c.ub, c.dsig, asd);
    // fv = -u' absv - ub vor' - rcpg (tv' piyb + tvdev pi_y) + VA(v'; sdb) + VA(vb; sd')
    f = afv[k];
    au[k] -= c.absv[k] * f;
    avor[k] -= c.ub[k] * f;
    atv[k] -= rcpg * c.piyb * f;
    py -= rcpg * tvdev * f;
    va_f_adj(k, K, f, c.sdb, c.dsig, av);
    va_s_adj(k, K, f, c.vb, c.dsig, asd);
    // ke = sum_l ww[k][l] (tv'_l - t'_l) + u' (ub + u0) + v' (vb + v0)
    const R e = ake[k];
    for (int l = 0; l < K; ++l) {
      atv[l] += c.ww[k * K + l] * e;
      at[l] -= c.ww[k * K + l] * e;
    }
    au[k] += (c.ub[k] + (c.u0 ? c.u0[k] : R(0))) * e;
    av[k] += (c.vb[k] + (c.v0 ? c.v0[k] : R(0))) * e;
    // yu = u' qb + ub q', yv = v' qb + vb q'
    au[k] += c.qb[k] * ayu[k];
    aq[k] += c.ub[k] * ayu[k];
    av[k] += c.qb[k] * ayv[k];
    aq[k] += c.vb[k] * ayv[k];
    // g = q' divb + qb div' + VA(q'; sdb) + VA(qb; sd')
    f = ag[k];
    aq[k] += c.divb[k] * f;
    adiv[k] += c.qb[k] * f;
    va_f_adj(k, K, f, c.sdb, c.dsig, aq);
    va_s_adj(k, K, f, c.qb, c.dsig, asd);
    // gt_pi = -sum_k dsig padv'
    apadv[k] -= c.dsig[k] * agtpi;
  }
  for (int k = 0; k < K; ++k) {
    // tv' = t' (1 + eps qb) + eps tb q'
    at[k] += (R(1) + c.eps * c.qb[k]) * atv[k];
    aq[k] += c.eps * c.tb[k] * atv[k];
    // x5' = alpha div' + wP padv' + w3 S[k+1]
    adiv[k] += c.alpha[k] * ax5[k];
    apadv[k] += c.wP[k] * ax5[k];
    aS[k + 1] += c.w3[k] * ax5[k];
  }
  // sd'[k] = sigm[k] S[0] - S[k] for 1 <= k <= K-1 (zero at both ends)
  for (int k = 1; k < K; ++k) {
    aS[0] += c.sigm[k] * asd[k];
    aS[k] -= asd[k];
  }
  // S[k] = sum_{l >= k} dsig_l (div' + padv')_l ; S[K] = 0
  R cum = R(0);
  for (int l = 0; l < K; ++l) {
    cum += aS[l];
    adiv[l] += c.dsig[l] * cum;
    apadv[l] += c.dsig[l] * cum;
  }
  // padv' = u' pixb + ub pi_x + v' piyb + vb pi_y
  for (int k = 0; k < K; ++k) {
    au[k] += c.pixb * apadv[k];
    av[k] += c.piyb * apadv[k];
    px += c.ub[k] * apadv[k];
    py += c.vb[k] * apadv[k];
  }
  *apix = px;
  *apiy = py;
}

// Operators of the implicit update for one total wavenumber n.
template <typename R>
struct ImplConst {
  int K;
  R dt, lap;                                  // time step, -n(n+1)/a^2
  const R *kv, *kd, *ktt, *kq;                // [K] at this n
  const R *ww, *tmtx, *gg, *dsig, *minv;      // [K][K], [K][K], [K], [K], [K][K] at this n
  const R* vd[4];                             // vertical diffusion of vor div t q, or null
  bool vd_skip_vordiv;                        // n < 2: no vertical diffusion of vor, div
};

// Adjoint of the implicit update of one coefficient, one real component
// (stride `st` between levels).  Inputs: adjoints of the new level
// an_* [K] and an_pi.  Outputs (overwritten): adjoints of the previous
// level ap_* and of the explicit tendencies aw_*.  Scratch: 4 K values.
template <typename R>
LBM_COL_HD void implicit_coef_adjoint(const ImplConst<R>& c, int st, const R* an_vor,
                                      const R* an_div, const R* an_t, const R* an_q, R an_pi,
                                      R* ap_vor, R* ap_div, R* ap_t, R* ap_q, R* ap_pi,
                                      R* aw_vor, R* aw_div, R* aw_t, R* aw_q, R* aw_pi,
                                      R* work) {
  const int K = c.K;
  const R dt = c.dt, dt2 = R(2) * dt;
  R* x = work;            // adjoint of a field before its vertical diffusion
  R* dbar = work + K;     // adjoint of the solved divergence
  R* rhs = work + 2 * K;  // adjoint of the right-hand side
  R* phy = work + 3 * K;  // adjoint of the geopotential term wdphiy
  const R* an[4] = {an_vor, an_div, an_t, an_q};
  R* ap[4] = {ap_vor, ap_div, ap_t, ap_q};
  R* aw[4] = {aw_vor, aw_div, aw_t, aw_q};
  for (int f = 0; f < 4; ++f) {
    // x = VD^T an  (no diffusion of vor, div at n < 2)
    const R* vd = c.vd[f];
    const bool use = vd && !(f < 2 && c.vd_skip_vordiv);
    for (int l = 0; l < K; ++l) {
      R s = R(0);
      if (use) {
        for (int k = 0; k < K; ++k) s += vd[k * K + l] * an[f][k * st];
      } else {
        s = an[f][l * st];
      }
      x[l] = s;
    }
    for (int k = 0; k < K; ++k) {
      const R v = x[k];
      if (f == 0 || f == 3) {
        // vor/q_new = (p + 2 dt w) / (1 + 2 dt kv|kq)
        const R r = R(1) / (R(1) + dt2 * (f == 0 ? c.kv[k] : c.kq[k]));
        ap[f][k * st] = v * r;
        aw[f][k * st] = dt2 * v * r;
      } else if (f == 1) {
        // d_new = 2 dbar - p_div
        dbar[k] = R(2) * v;
        ap[f][k * st] = -v;
      } else {
        // t_new = (p_t + 2 dt (w_t - tmtx dbar)) / ft
        const R ft = R(1) + dt2 * c.ktt[k];
        ap[f][k * st] = v / ft;
        aw[f][k * st] = dt2 * v / ft;
      }
    }
  }
  // pi_new = p_pi + 2 dt (w_pi - sum dsig dbar)
  *ap_pi = an_pi;
  *aw_pi = dt2 * an_pi;
  for (int l = 0; l < K; ++l) {
    R s = R(0);
    for (int k = 0; k < K; ++k) s -= c.tmtx[k * K + l] * aw_t[k * st];
    dbar[l] += s - c.dsig[l] * (*aw_pi);
  }
  // dbar = Minv rhs
  for (int l = 0; l < K; ++l) {
    R s = R(0);
    for (int k = 0; k < K; ++k) s += c.minv[k * K + l] * dbar[k];
    rhs[l] = s;
  }
  // rhs = p_div (1 + dt kd) ft + dt (w_div ft - lap wdphiy)
  R apix = R(0);
  for (int k = 0; k < K; ++k) {
    const R ft = R(1) + dt2 * c.ktt[k];
    ap_div[k * st] += (R(1) + dt * c.kd[k]) * ft * rhs[k];
    aw_div[k * st] = dt * ft * rhs[k];
    phy[k] = -dt * c.lap * rhs[k];
    // wdphiy = WW wdx + gg ft (p_pi + dt w_pi)
    apix += c.gg[k] * ft * phy[k];
  }
  *ap_pi += apix;
  *aw_pi += dt * apix;
  // wdx = p_t (1 + dt ktt) + dt w_t
  for (int l = 0; l < K; ++l) {
    R s = R(0);
    for (int k = 0; k < K; ++k) s += c.ww[k * K + l] * phy[k];
    ap_t[l * st] += (R(1) + dt * c.ktt[l]) * s;
    aw_t[l * st] += dt * s;
  }
}

}  // namespace lbm_adj
