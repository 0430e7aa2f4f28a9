// Reference-layout kernels of the time step: the grid-point part of
// Dynamics.tendencies (dynamics.py:176-267) and Integrator.step
// (integrator.py:264-315).  The fused ensemble stepper (stepper.cu) runs the
// same algebra on its own layouts; these serve the drop-in API
// (Dynamics.tendencies / Integrator.step called directly, the forward
// start of LBM.run on an arbitrary grid state).
#include "lbm_common.cuh"

namespace lbm {

constexpr int KMAX_LOCAL = 64;   // largest level count the column kernels hold

// Vertical advection, SECOND_CENTERED ADVECTIVE_FORM with the overall +
// sign of dynamics.py:117-143; f(l), s(l) are level accessors.
template <typename R, typename F, typename S>
LBM_D R vert_adv(int k, int K, F f, S s, R dsk) {
  const R fk = f(k);
  const R flo = (k >= 1) ? s(k) * R(0.5) * (fk + f(k - 1)) : R(0);
  const R fhi = (k + 1 <= K - 1) ? s(k + 1) * R(0.5) * (f(k + 1) + fk) : R(0);
  return (fhi - flo - fk * (s(k + 1) - s(k))) / dsk;
}

template <typename R>
__global__ void k_tendency_grid(lbm_tend_grid_args a) {
  const int J = a.nlat, I = a.nlon, K = a.kmax;
  const size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t ncol2 = (size_t)J * I;
  if (col >= (size_t)a.nmem * ncol2) return;
  const size_t e = col / ncol2, ji = col % ncol2;
  const R kappa = R(a.kappa), eps = R(a.epsvt), rair = R(a.rair);
  auto P = [](const void* p) { return (const R*)p; };
  const R *dsig = P(a.dsig), *sigm = P(a.sigm), *alpha = P(a.alpha), *w3 = P(a.w3),
          *wP = P(a.wP), *cpg = P(a.cpg), *sig = P(a.sig), *ww = P(a.ww), *tmtx = P(a.tmtx),
          *tref = P(a.tref);
  const size_t b3 = ji * K;                // basic-state column offset
  const size_t p3 = col * K;               // perturbation column offset
  const R *ub = P(a.ub) + b3, *vb = P(a.vb) + b3, *tb = P(a.tb) + b3, *qb = P(a.qb) + b3,
          *tvb = P(a.tvb) + b3, *absv = P(a.absvor) + b3, *divb = P(a.divb) + b3,
          *x5b = P(a.x5b) + b3, *sdb = P(a.sdotb) + ji * (K + 1);
  const R *u = P(a.u) + p3, *v = P(a.v) + p3, *t = P(a.t) + p3, *q = P(a.q) + p3,
          *vor = P(a.vor) + p3, *div = P(a.div) + p3;
  const R pixb = P(a.pixb)[ji], piyb = P(a.piyb)[ji], psb = P(a.psb)[ji];
  const R pix = P(a.pix)[col], piy = P(a.piy)[col], ps = P(a.ps)[col];

  R S[KMAX_LOCAL + 1], sd[KMAX_LOCAL + 1], padv[KMAX_LOCAL], x[KMAX_LOCAL];
  for (int k = 0; k < K; ++k) padv[k] = u[k] * pixb + ub[k] * pix + v[k] * piyb + vb[k] * piy;
  // S[k] = sum_{l>=k} dsig_l (div + padv)_l  (dynamics.py:96-102)
  S[K] = R(0);
  for (int k = K - 1; k >= 0; --k) S[k] = S[k + 1] + (div[k] + padv[k]) * dsig[k];
  for (int k = 0; k <= K; ++k) sd[k] = sigm[k] * S[0] - S[k];   // dynamics.py:105-114
  sd[0] = R(0);
  sd[K] = R(0);
  // gt_pi = -S[0] + sum dsig div (dynamics.py:188) = -sum dsig padv: summed
  // directly, without the cancellation of two O(div) terms
  R gtpi = R(0);
  for (int k = 0; k < K; ++k) gtpi -= padv[k] * dsig[k];
  if (a.frc_ps) gtpi += P(a.frc_ps)[e * a.frc_ps_stride + ji];
  ((R*)a.gt_pi)[col] = gtpi;
  for (int k = 0; k < K; ++k) x[k] = t[k] + eps * (t[k] * qb[k] + tb[k] * q[k]);  // tv'

  R *fu = (R*)a.fu + p3, *fv = (R*)a.fv + p3, *ke = (R*)a.ke + p3, *gt = (R*)a.gt + p3,
    *xu = (R*)a.xu + p3, *xv = (R*)a.xv + p3, *g = (R*)a.g + p3, *yu = (R*)a.yu + p3,
    *yv = (R*)a.yv + p3;
  const R* frt = a.frc_t ? P(a.frc_t) + e * a.frc_t_stride + b3 : nullptr;
  const R* frq = a.frc_q ? P(a.frc_q) + e * a.frc_q_stride + b3 : nullptr;
  auto fS = [&](int l) { return sd[l]; };
  auto fSb = [&](int l) { return sdb[l]; };
  for (int k = 0; k < K; ++k) {
    const R tv = x[k];
    const R x5p = alpha[k] * div[k] + wP[k] * padv[k] + w3[k] * S[k + 1];
    const R adiab = -kappa * (tv * x5b[k] + tvb[k] * x5p);
    const R tdev = tb[k] - tref[k];
    xu[k] = u[k] * tdev + ub[k] * t[k];
    xv[k] = v[k] * tdev + vb[k] * t[k];
    const R hadv = t[k] * divb[k] + tdev * div[k];
    const R vadv = vert_adv<R>(k, K, [&](int l) { return t[l]; }, fSb, dsig[k]) +
                   vert_adv<R>(k, K, [&](int l) { return tb[l]; }, fS, dsig[k]);
    R tm = R(0);
    for (int l = 0; l < K; ++l) tm += div[l] * tmtx[k * K + l];
    R gtk = adiab + hadv + vadv + tm;
    if (frt) gtk += frt[k];
    gt[k] = gtk;
    // momentum (dynamics.py:224-237)
    const R rcpg = rair * cpg[k];
    const R tvdev = tvb[k] - tref[k];
    R fuk = v[k] * absv[k] + vb[k] * vor[k];
    R fvk = -u[k] * absv[k] - ub[k] * vor[k];
    fuk -= rcpg * (tv * pixb + tvdev * pix);
    fvk -= rcpg * (tv * piyb + tvdev * piy);
    fuk += vert_adv<R>(k, K, [&](int l) { return u[l]; }, fSb, dsig[k]) +
           vert_adv<R>(k, K, [&](int l) { return ub[l]; }, fS, dsig[k]);
    fvk += vert_adv<R>(k, K, [&](int l) { return v[l]; }, fSb, dsig[k]) +
           vert_adv<R>(k, K, [&](int l) { return vb[l]; }, fS, dsig[k]);
    fu[k] = fuk;
    fv[k] = fvk;
    R phiv = R(0);
    for (int l = 0; l < K; ++l) phiv += (x[l] - t[l]) * ww[k * K + l];
    R kek = phiv + u[k] * ub[k] + v[k] * vb[k];
    if (a.lin_u)   // tangent-linear: linearised about the trajectory (lin_u, lin_v)
      kek += P(a.lin_u)[p3 + k] * u[k] + P(a.lin_v)[p3 + k] * v[k];
    else if (!a.strictly_linear)
      kek += R(0.5) * (u[k] * u[k] + v[k] * v[k]);
    ke[k] = kek;
    // humidity (dynamics.py:256-262)
    yu[k] = u[k] * qb[k] + ub[k] * q[k];
    yv[k] = v[k] * qb[k] + vb[k] * q[k];
    R gk = q[k] * divb[k] + qb[k] * div[k] +
           vert_adv<R>(k, K, [&](int l) { return q[l]; }, fSb, dsig[k]) +
           vert_adv<R>(k, K, [&](int l) { return qb[l]; }, fS, dsig[k]);
    if (frq) gk += frq[k];
    g[k] = gk;
    if (a.omega) ((R*)a.omega)[p3 + k] = -sig[k] * (x5p * psb + x5b[k] * ps);
  }
  if (a.sdot)
    for (int k = 0; k <= K; ++k) ((R*)a.sdot)[col * (K + 1) + k] = sd[k];
}

// One block per (e, m, n) coefficient, thread per level.
template <typename R>
__global__ void k_implicit_rect(lbm_implicit_args a) {
  const int K = a.kmax, M = a.nmax + 1;
  const int n = blockIdx.x, m = blockIdx.y, e = blockIdx.z, k = threadIdx.x;
  __shared__ C2<R> sx[KMAX_LOCAL], sy[KMAX_LOCAL];
  const size_t o3 = (((size_t)e * M + m) * M + n) * K + k;
  const size_t o2 = ((size_t)e * M + m) * M + n;
  auto P = [](const void* p) { return (const R*)p; };
  C2<R>* nv = (C2<R>*)a.n_vor;
  C2<R>* nd = (C2<R>*)a.n_div;
  C2<R>* nt = (C2<R>*)a.n_t;
  C2<R>* nq = (C2<R>*)a.n_q;
  C2<R>* np = (C2<R>*)a.n_pi;
  const C2<R> z = cmk<R>(0, 0);
  if (n < m) {                      // outside the triangle: keep zeros
    if (k < K) { nv[o3] = z; nd[o3] = z; nt[o3] = z; nq[o3] = z; }
    if (k == 0) np[o2] = z;
    return;
  }
  const R dt = R(a.dt), dt2 = R(2) * dt;
  const R ktt = P(a.ktt)[n * K + k], kd = P(a.kd)[n * K + k];
  const R kv = P(a.kv)[n * K + k], kq = P(a.kq)[n * K + k];
  const R ft = R(1) + dt2 * ktt;
  const R lap = P(a.lap)[n];
  const C2<R> pt = ((const C2<R>*)a.p_t)[o3], wtt = ((const C2<R>*)a.w_t)[o3];
  // wdx = T(t-dt)(1 + dt ktt) + dt wt_t ; wdphix = WW wdx  (integrator.py:287-288)
  sx[k] = pt * (R(1) + dt * ktt) + wtt * dt;
  __syncthreads();
  C2<R> wdphix = z;
  for (int l = 0; l < K; ++l) cfma(wdphix, P(a.ww)[k * K + l], sx[l]);
  const C2<R> ppi = ((const C2<R>*)a.p_pi)[o2], wpi = ((const C2<R>*)a.w_pi)[o2];
  const C2<R> wdpix = ppi + wpi * dt;
  const C2<R> wdphiy = wdphix + wdpix * (ft * P(a.gg)[k]);
  const C2<R> pdv = ((const C2<R>*)a.p_div)[o3], wdv = ((const C2<R>*)a.w_div)[o3];
  const C2<R> rhs = pdv * ((R(1) + dt * kd) * ft) + (wdv * ft - wdphiy * lap) * dt;
  __syncthreads();
  sy[k] = rhs;
  __syncthreads();
  C2<R> dbar = z;
  const R* mi = P(a.minv) + (size_t)n * K * K;
  for (int l = 0; l < K; ++l) cfma(dbar, mi[k * K + l], sy[l]);
  __syncthreads();
  sx[k] = dbar;
  __syncthreads();
  C2<R> corr = z, dsum = z;
  for (int l = 0; l < K; ++l) {
    cfma(corr, P(a.tmtx)[k * K + l], sx[l]);
    cfma(dsum, P(a.dsig)[l], sx[l]);
  }
  const C2<R> wt2 = wtt - corr;
  const C2<R> wpi2 = wpi - dsum;
  const C2<R> pv = ((const C2<R>*)a.p_vor)[o3], wv = ((const C2<R>*)a.w_vor)[o3];
  const C2<R> pq = ((const C2<R>*)a.p_q)[o3], wq = ((const C2<R>*)a.w_q)[o3];
  C2<R> v_new = (pv + wv * dt2) * (R(1) / (R(1) + dt2 * kv));
  C2<R> d_new = dbar * R(2) - pdv;
  C2<R> t_new = (pt + wt2 * dt2) * (R(1) / ft);
  C2<R> q_new = (pq + wq * dt2) * (R(1) / (R(1) + dt2 * kq));
  if (k == 0) np[o2] = ppi + wpi2 * dt2;
  // implicit vertical diffusion (integrator.py:311-314), n = 0, 1 skipped for vor/div
  const void* vd[4] = {a.vd_vor, a.vd_div, a.vd_t, a.vd_q};
  C2<R>* vals[4] = {&v_new, &d_new, &t_new, &q_new};
  for (int f = 0; f < 4; ++f) {
    if (!vd[f]) continue;
    if (f < 2 && n < 2) continue;
    __syncthreads();
    sx[k] = *vals[f];
    __syncthreads();
    C2<R> o = z;
    for (int l = 0; l < K; ++l) cfma(o, P(vd[f])[k * K + l], sx[l]);
    *vals[f] = o;
  }
  nv[o3] = v_new;
  nd[o3] = d_new;
  nt[o3] = t_new;
  nq[o3] = q_new;
}

}  // namespace lbm

using namespace lbm;

extern "C" {

int lbm_tendency_grid(int prec, const lbm_tend_grid_args* a, void* stream) {
  if (!a || a->nmem < 1 || a->kmax < 1 || a->kmax > KMAX_LOCAL || a->nlat < 2 || a->nlon < 2)
    return LBM_ERR_ARG;
  if ((a->lin_u == nullptr) != (a->lin_v == nullptr)) return LBM_ERR_ARG;
  const size_t cols = (size_t)a->nmem * a->nlat * a->nlon;
  const int threads = 32;   // one member's 8192 columns (T42) over all SMs
  const unsigned blocks = (unsigned)((cols + threads - 1) / threads);
  if (prec == LBM_F64)
    k_tendency_grid<double><<<blocks, threads, 0, (cudaStream_t)stream>>>(*a);
  else if (prec == LBM_F32)
    k_tendency_grid<float><<<blocks, threads, 0, (cudaStream_t)stream>>>(*a);
  else
    return LBM_ERR_ARG;
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

int lbm_implicit_step(int prec, const lbm_implicit_args* a, void* stream) {
  if (!a || a->nmem < 1 || a->kmax < 1 || a->kmax > KMAX_LOCAL || a->nmax < 1) return LBM_ERR_ARG;
  const int M = a->nmax + 1;
  dim3 grid(M, M, a->nmem);
  if (prec == LBM_F64)
    k_implicit_rect<double><<<grid, a->kmax, 0, (cudaStream_t)stream>>>(*a);
  else if (prec == LBM_F32)
    k_implicit_rect<float><<<grid, a->kmax, 0, (cudaStream_t)stream>>>(*a);
  else
    return LBM_ERR_ARG;
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

}  // extern "C"
