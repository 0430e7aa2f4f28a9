// Host build of the adjoint column arithmetic (lbm_isca_gb300/csrc/
// adjoint_col.cuh) for the CPU tests: the same source the device kernels
// compile, exposed through plain C entry points.
#include "../lbm_isca_gb300/csrc/adjoint_col.cuh"

extern "C" {

// vert: dsig sigm alpha w3 wP cpg ww tmtx tref; bs: ub vb tb qb tvb absv divb x5b sdb
// ain: fu fv ke gt xu xv g yu yv; aout: u v t q vor div
void host_tendency_column_adjoint(int K, double kappa, double eps, double rair,
                                  const double* const* vert, const double* const* bs,
                                  double pixb, double piyb, const double* u0,
                                  const double* v0, const double* const* ain, double agtpi,
                                  double* const* aout, double* apix, double* apiy,
                                  double* work) {
  lbm_adj::ColConst<double> c;
  c.K = K;
  c.kappa = kappa;
  c.eps = eps;
  c.rair = rair;
  c.dsig = vert[0]; c.sigm = vert[1]; c.alpha = vert[2]; c.w3 = vert[3]; c.wP = vert[4];
  c.cpg = vert[5]; c.ww = vert[6]; c.tmtx = vert[7]; c.tref = vert[8];
  c.ub = bs[0]; c.vb = bs[1]; c.tb = bs[2]; c.qb = bs[3]; c.tvb = bs[4]; c.absv = bs[5];
  c.divb = bs[6]; c.x5b = bs[7]; c.sdb = bs[8];
  c.pixb = pixb;
  c.piyb = piyb;
  c.u0 = u0;
  c.v0 = v0;
  lbm_adj::tendency_column_adjoint<double>(c, ain[0], ain[1], ain[2], ain[3], ain[4], ain[5],
                                           ain[6], ain[7], ain[8], agtpi, aout[0], aout[1],
                                           aout[2], aout[3], aout[4], aout[5], apix, apiy,
                                           work);
}

// ops: kv kd ktt kq ww tmtx gg dsig minv (at one n); vd: vor div t q (or null)
// an/ap/aw: vor div t q; stride 1 (one real component)
void host_implicit_coef_adjoint(int K, double dt, double lap, const double* const* ops,
                                const double* const* vd, int skip_vordiv,
                                const double* const* an, double an_pi, double* const* ap,
                                double* ap_pi, double* const* aw, double* aw_pi,
                                double* work) {
  lbm_adj::ImplConst<double> c;
  c.K = K;
  c.dt = dt;
  c.lap = lap;
  c.kv = ops[0]; c.kd = ops[1]; c.ktt = ops[2]; c.kq = ops[3]; c.ww = ops[4];
  c.tmtx = ops[5]; c.gg = ops[6]; c.dsig = ops[7]; c.minv = ops[8];
  for (int f = 0; f < 4; ++f) c.vd[f] = vd[f];
  c.vd_skip_vordiv = skip_vordiv != 0;
  lbm_adj::implicit_coef_adjoint<double>(c, 1, an[0], an[1], an[2], an[3], an_pi, ap[0], ap[1],
                                         ap[2], ap[3], ap_pi, aw[0], aw[1], aw[2], aw[3], aw_pi,
                                         work);
}

}  // extern "C"
