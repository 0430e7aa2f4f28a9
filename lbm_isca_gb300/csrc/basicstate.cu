// Basic-state preprocessing on the device, one thread per grid column (FP64):
// surface pressure from geopotential height (basicstate.py:115-151), natural
// cubic spline interpolation in ln p (basicstate.py:176-238; Press et al.,
// Numerical Recipes, sect. 3.3) for the pressure -> sigma step
// (basicstate.py:241-260), and the zonal-mean / stationary-wave filter
// (basicstate.py:165-173).  Batched over any number of columns, so many
// basic states (months, years) are prepared in one launch.

#include "lbm_common.cuh"

namespace lbm {

constexpr int BS_MAXLEV = 64;     // pressure levels a column may have

// ps = exp(ln p_{k-1} + (ln p_k - ln p_{k-1}) (zs - z_{k-1}) / (z_k - z_{k-1}))
// at k = the lowest level whose height exceeds zs (the top level if none),
// kept within [1, nk - 1].
__global__ void k_z2ps(long long ncol, int nk, const double* __restrict__ z,
                       const double* __restrict__ zs, const double* __restrict__ plev,
                       double* __restrict__ ps) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncol;
       c += (long long)gridDim.x * blockDim.x) {
    const double* zc = z + c * nk;
    const double s = zs ? zs[c] : 0.0;
    int ka = nk - 1;
    for (int k = 0; k < nk; ++k)
      if (zc[k] > s) { ka = k; break; }
    ka = ka < 1 ? 1 : ka;
    const double l0 = log(plev[ka - 1]), l1 = log(plev[ka]);
    const double zk = zc[ka], zkm = zc[ka - 1];
    ps[c] = exp(l0 + (l1 - l0) * (s - zkm) / (zk - zkm));
  }
}

// Natural cubic spline through (x_k, z_ck), x shared and monotonic, evaluated
// at xi_cl.  Second derivatives by the tridiagonal sweep with zero end
// curvature; outside [x_0, x_{nk-1}] the end value (or xmiss when asked).
__global__ void k_spline(long long ncol, int nk, int nl, const double* __restrict__ x,
                         const double* __restrict__ z, const double* __restrict__ xi,
                         double* __restrict__ out, int omisb, int omist, double xmiss) {
  const bool desc = x[nk - 1] < x[0];
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncol;
       c += (long long)gridDim.x * blockDim.x) {
    const double* zc = z + c * nk;
    double y2[BS_MAXLEV], uu[BS_MAXLEV], dg[BS_MAXLEV];
    dg[0] = 0.0;
    uu[0] = 0.0;
    for (int i = 1; i < nk - 1; ++i) {
      const double sg = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
      const double p = sg * dg[i - 1] + 2.0;
      dg[i] = (sg - 1.0) / p;
      const double slope = (zc[i + 1] - zc[i]) / (x[i + 1] - x[i]) -
                           (zc[i] - zc[i - 1]) / (x[i] - x[i - 1]);
      uu[i] = (6.0 * slope / (x[i + 1] - x[i - 1]) - sg * uu[i - 1]) / p;
    }
    y2[nk - 1] = 0.0;
    for (int i = nk - 2; i >= 0; --i) y2[i] = dg[i] * y2[i + 1] + uu[i];
    for (int l = 0; l < nl; ++l) {
      const double t = xi[c * nl + l];
      // ku = number of abscissae at or before t in the direction of x
      int ku = 0;
      for (int k = 0; k < nk; ++k)
        if (desc ? (x[k] >= t) : (x[k] <= t)) ku = k + 1;
      double v;
      if (ku == 0) {
        v = omisb ? xmiss : zc[0];
      } else if (ku == nk) {
        v = omist ? xmiss : zc[nk - 1];
      } else {
        const int kc = ku;
        const double h = x[kc] - x[kc - 1];
        const double a = (x[kc] - t) / h, b = (t - x[kc - 1]) / h;
        v = a * zc[kc - 1] + b * zc[kc] +
            (a * (a * a - 1.0) * y2[kc - 1] + b * (b * b - 1.0) * y2[kc]) * h * h / 6.0;
      }
      out[c * nl + l] = v;
    }
  }
}

// mode 1: every value -> its zonal mean; mode 2: minus its zonal mean.
// x [nlat][nlon][nk]; one thread per (latitude, k).
__global__ void k_zonal_filter(int nlat, int nlon, int nk, double* __restrict__ x, int mode) {
  const long long n = (long long)nlat * nk;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    const long long j = r / nk, k = r - j * nk;
    double* row = x + j * (long long)nlon * nk + k;
    double s = 0.0;
    for (int i = 0; i < nlon; ++i) s += row[(long long)i * nk];
    const double mean = s / nlon;
    for (int i = 0; i < nlon; ++i) row[(long long)i * nk] = mode == 1 ? mean : row[(long long)i * nk] - mean;
  }
}

inline unsigned col_blocks(long long n) {
  long long b = (n + 127) / 128;
  return (unsigned)(b > 8192 ? 8192 : (b < 1 ? 1 : b));
}

}  // namespace lbm

using namespace lbm;

extern "C" {

int lbm_z2ps(int64_t ncol, int nk, const double* z, const double* zs, const double* plev,
             double* ps, void* stream) {
  if (ncol < 1 || nk < 2 || !z || !plev || !ps) return LBM_ERR_ARG;
  k_z2ps<<<col_blocks(ncol), 128, 0, (cudaStream_t)stream>>>(ncol, nk, z, zs, plev, ps);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

int lbm_spline(int64_t ncol, int nk, int nl, const double* x, const double* z, const double* xi,
               double* out, int omisb, int omist, double xmiss, void* stream) {
  if (ncol < 1 || nk < 2 || nk > BS_MAXLEV || nl < 1 || !x || !z || !xi || !out)
    return LBM_ERR_ARG;
  k_spline<<<col_blocks(ncol), 128, 0, (cudaStream_t)stream>>>(ncol, nk, nl, x, z, xi, out,
                                                                omisb, omist, xmiss);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

int lbm_zonal_filter(int nlat, int nlon, int nk, double* x, int mode, void* stream) {
  if (nlat < 1 || nlon < 1 || nk < 1 || !x || (mode != 1 && mode != 2)) return LBM_ERR_ARG;
  k_zonal_filter<<<col_blocks((long long)nlat * nk), 128, 0, (cudaStream_t)stream>>>(nlat, nlon,
                                                                                   nk, x, mode);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

}  // extern "C"
