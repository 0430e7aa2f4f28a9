// Adjoint kernels of the reference-layout time step: the transposes of
// lbm_tendency_grid (grid-point part of Dynamics.tendencies, reference
// dynamics.py:176-267) and of lbm_implicit_step (Integrator.step,
// integrator.py:264-315).  The spectral transforms need no kernels of their
// own: the transpose of each transform is another transform of the library
// with rescaled tables.  The column arithmetic lives in adjoint_col.cuh.
#include "lbm_common.cuh"
#include "adjoint_col.cuh"

namespace lbm {

// 32-thread blocks: one member's columns (8192 at T42) or coefficients
// (3698) spread over all SMs instead of filling a few.
constexpr int ADJ_THREADS = 32;

// One thread per grid column (member, latitude, longitude).
template <typename R, int KM>
__global__ void __launch_bounds__(ADJ_THREADS) k_tendency_grid_adj(lbm_tend_adj_args a) {
  const int J = a.nlat, I = a.nlon, K = a.kmax;
  const size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t ncol2 = (size_t)J * I;
  if (col >= (size_t)a.nmem * ncol2) return;
  const size_t ji = col % ncol2;
  auto P = [](const void* p) { return (const R*)p; };
  const size_t b3 = ji * K, p3 = col * K;
  lbm_adj::ColConst<R> c;
  c.K = K;
  c.kappa = R(a.kappa);
  c.eps = R(a.epsvt);
  c.rair = R(a.rair);
  c.dsig = P(a.dsig);
  c.sigm = P(a.sigm);
  c.alpha = P(a.alpha);
  c.w3 = P(a.w3);
  c.wP = P(a.wP);
  c.cpg = P(a.cpg);
  c.ww = P(a.ww);
  c.tmtx = P(a.tmtx);
  c.tref = P(a.tref);
  c.ub = P(a.ub) + b3;
  c.vb = P(a.vb) + b3;
  c.tb = P(a.tb) + b3;
  c.qb = P(a.qb) + b3;
  c.tvb = P(a.tvb) + b3;
  c.absv = P(a.absvor) + b3;
  c.divb = P(a.divb) + b3;
  c.x5b = P(a.x5b) + b3;
  c.sdb = P(a.sdotb) + ji * (K + 1);
  c.pixb = P(a.pixb)[ji];
  c.piyb = P(a.piyb)[ji];
  c.u0 = a.u0 ? P(a.u0) + p3 : nullptr;
  c.v0 = a.v0 ? P(a.v0) + p3 : nullptr;
  R work[5 * (KM + 1)];
  // the adjoints are accumulated level by level (K x K scatters of the
  // hydrostatic and tmtx transposes, the vertical-advection transposes):
  // into thread-local arrays, whose elements the hardware interleaves across
  // the threads of a warp, and written to the level-strided outputs once
  R lu[KM], lv[KM], lt[KM], lq[KM], lvor[KM], ldiv[KM];
  lbm_adj::tendency_column_adjoint<R>(
      c, P(a.a_fu) + p3, P(a.a_fv) + p3, P(a.a_ke) + p3, P(a.a_gt) + p3, P(a.a_xu) + p3,
      P(a.a_xv) + p3, P(a.a_g) + p3, P(a.a_yu) + p3, P(a.a_yv) + p3, P(a.a_gt_pi)[col],
      lu, lv, lt, lq, lvor, ldiv, (R*)a.a_pix + col, (R*)a.a_piy + col, work);
  R *ou = (R*)a.a_u + p3, *ov = (R*)a.a_v + p3, *ot = (R*)a.a_t + p3, *oq = (R*)a.a_q + p3,
    *ovor = (R*)a.a_vor + p3, *odiv = (R*)a.a_div + p3;
  for (int k = 0; k < K; ++k) {
    ou[k] = lu[k];
    ov[k] = lv[k];
    ot[k] = lt[k];
    oq[k] = lq[k];
    ovor[k] = lvor[k];
    odiv[k] = ldiv[k];
  }
}

// One thread per (member, m, n, real/imaginary part).
template <typename R, int KM>
__global__ void __launch_bounds__(ADJ_THREADS) k_implicit_adj(lbm_implicit_adj_args a) {
  const int K = a.kmax, M = a.nmax + 1;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)a.nmem * M * M * 2;
  if (idx >= total) return;
  const int comp = (int)(idx & 1);
  const size_t coef = idx >> 1;                 // (e, m, n)
  const int n = (int)(coef % M), m = (int)((coef / M) % M);
  auto P = [](const void* p) { return (const R*)p; };
  const size_t o3 = coef * K * 2 + comp, o2 = coef * 2 + comp;
  R* ap[5] = {(R*)a.ap_vor + o3, (R*)a.ap_div + o3, (R*)a.ap_t + o3, (R*)a.ap_q + o3,
              (R*)a.ap_pi + o2};
  R* aw[5] = {(R*)a.aw_vor + o3, (R*)a.aw_div + o3, (R*)a.aw_t + o3, (R*)a.aw_q + o3,
              (R*)a.aw_pi + o2};
  if (n < m) {           // outside the triangle the update writes zeros
    for (int f = 0; f < 4; ++f)
      for (int k = 0; k < K; ++k) ap[f][2 * k] = aw[f][2 * k] = R(0);
    *ap[4] = *aw[4] = R(0);
    return;
  }
  lbm_adj::ImplConst<R> c;
  c.K = K;
  c.dt = R(a.dt);
  c.lap = P(a.lap)[n];
  c.kv = P(a.kv) + (size_t)n * K;
  c.kd = P(a.kd) + (size_t)n * K;
  c.ktt = P(a.ktt) + (size_t)n * K;
  c.kq = P(a.kq) + (size_t)n * K;
  c.ww = P(a.ww);
  c.tmtx = P(a.tmtx);
  c.gg = P(a.gg);
  c.dsig = P(a.dsig);
  c.minv = P(a.minv) + (size_t)n * K * K;
  c.vd[0] = P(a.vd_vor);
  c.vd[1] = P(a.vd_div);
  c.vd[2] = P(a.vd_t);
  c.vd[3] = P(a.vd_q);
  c.vd_skip_vordiv = n < 2;
  R work[4 * KM];
  lbm_adj::implicit_coef_adjoint<R>(c, 2, P(a.an_vor) + o3, P(a.an_div) + o3, P(a.an_t) + o3,
                                    P(a.an_q) + o3, P(a.an_pi)[o2], ap[0], ap[1], ap[2], ap[3],
                                    ap[4], aw[0], aw[1], aw[2], aw[3], aw[4], work);
}

template <typename R>
static int tend_adj(const lbm_tend_adj_args* a, cudaStream_t st) {
  const size_t cols = (size_t)a->nmem * a->nlat * a->nlon;
  const unsigned blocks = (unsigned)((cols + ADJ_THREADS - 1) / ADJ_THREADS);
  if (a->kmax <= 32)
    k_tendency_grid_adj<R, 32><<<blocks, ADJ_THREADS, 0, st>>>(*a);
  else
    k_tendency_grid_adj<R, 64><<<blocks, ADJ_THREADS, 0, st>>>(*a);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

template <typename R>
static int impl_adj(const lbm_implicit_adj_args* a, cudaStream_t st) {
  const size_t M = (size_t)a->nmax + 1;
  const size_t total = (size_t)a->nmem * M * M * 2;
  const unsigned blocks = (unsigned)((total + ADJ_THREADS - 1) / ADJ_THREADS);
  if (a->kmax <= 32)
    k_implicit_adj<R, 32><<<blocks, ADJ_THREADS, 0, st>>>(*a);
  else
    k_implicit_adj<R, 64><<<blocks, ADJ_THREADS, 0, st>>>(*a);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

}  // namespace lbm

using namespace lbm;

extern "C" {

int lbm_tendency_grid_adjoint(int prec, const lbm_tend_adj_args* a, void* stream) {
  if (!a || a->nmem < 1 || a->kmax < 1 || a->kmax > 64 || a->nlat < 2 || a->nlon < 2)
    return LBM_ERR_ARG;
  const void* need[] = {a->dsig,  a->sigm, a->alpha, a->w3,    a->wP,    a->cpg,   a->ww,
                        a->tmtx,  a->tref, a->ub,    a->vb,    a->tb,    a->qb,    a->tvb,
                        a->absvor, a->divb, a->x5b,  a->sdotb, a->pixb,  a->piyb,  a->a_fu,
                        a->a_fv,  a->a_ke, a->a_gt,  a->a_xu,  a->a_xv,  a->a_g,   a->a_yu,
                        a->a_yv,  a->a_gt_pi, a->a_u, a->a_v,  a->a_t,   a->a_q,   a->a_vor,
                        a->a_div, a->a_pix, a->a_piy};
  for (const void* p : need)
    if (!p) return LBM_ERR_ARG;
  if ((a->u0 == nullptr) != (a->v0 == nullptr)) return LBM_ERR_ARG;
  if (prec == LBM_F64) return tend_adj<double>(a, (cudaStream_t)stream);
  if (prec == LBM_F32) return tend_adj<float>(a, (cudaStream_t)stream);
  return LBM_ERR_ARG;
}

int lbm_implicit_step_adjoint(int prec, const lbm_implicit_adj_args* a, void* stream) {
  if (!a || a->nmem < 1 || a->kmax < 1 || a->kmax > 64 || a->nmax < 1) return LBM_ERR_ARG;
  const void* need[] = {a->lap,    a->kv,     a->kd,    a->ktt,    a->kq,     a->ww,
                        a->tmtx,   a->gg,     a->dsig,  a->minv,   a->an_vor, a->an_div,
                        a->an_t,   a->an_pi,  a->an_q,  a->ap_vor, a->ap_div, a->ap_t,
                        a->ap_pi,  a->ap_q,   a->aw_vor, a->aw_div, a->aw_t,  a->aw_pi,
                        a->aw_q};
  for (const void* p : need)
    if (!p) return LBM_ERR_ARG;
  if (prec == LBM_F64) return impl_adj<double>(a, (cudaStream_t)stream);
  if (prec == LBM_F32) return impl_adj<float>(a, (cudaStream_t)stream);
  return LBM_ERR_ARG;
}

}  // extern "C"
