// One-off FP64 setup kernels: Gaussian grid, Legendre tables, FFT twiddles,
// semi-implicit matrices and their batched inverse.  These replace the
// host-side numpy setup of the reference (spectral.py:58-154,
// integrator.py:130-163, 216-228) so the whole model is built on the device.
#include "lbm_common.cuh"

namespace lbm {

// Gauss-Legendre nodes by Newton iteration on P_nlat (three-term
// recurrence), one thread per northern node; the southern half is mirrored
// and the weights are renormalised to sum to exactly one, as
// numpy.polynomial.legendre.leggauss symmetrises and rescales its result.
__global__ void k_gauss_legendre(int nlat, double* mu, double* gw) {
  extern __shared__ double wsum[];
  const int i = threadIdx.x;
  const int half = (nlat + 1) / 2;
  double x = 0.0, w = 0.0;
  if (i < half) {
    x = cospi((i + 0.75) / (nlat + 0.5));
    double dp = 1.0;
    int extra = 2;                 // two more steps once |dx| < 1e-14
    for (int it = 0; it < 100 && extra > 0; ++it) {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= nlat; ++k) {
        double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      // P'_n(x) = n (x P_n - P_{n-1}) / (x^2 - 1)
      dp = nlat * (x * p1 - p0) / (x * x - 1.0);
      const double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-14) --extra;
    }
    {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= nlat; ++k) {
        double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = nlat * (x * p1 - p0) / (x * x - 1.0);
    }
    if ((nlat & 1) && i == half - 1) x = 0.0;
    w = 1.0 / ((1.0 - x * x) * dp * dp);  // = (Gauss weight) / 2
    mu[i] = x;
    gw[i] = w;
    mu[nlat - 1 - i] = -x;
    gw[nlat - 1 - i] = w;
  }
  __syncthreads();
  if (i == 0) {
    double s = 0.0;
    for (int j = 0; j < nlat; ++j) s += gw[j];
    wsum[0] = s;
  }
  __syncthreads();
  for (int j = i; j < nlat; j += blockDim.x) gw[j] = gw[j] / wsum[0];
}

// Fully normalised P_n^m and H_n^m = (1 - mu^2) dP/dmu; one thread per
// (m, j).  Same recurrences and operation order as spectral.py:102-138.
__global__ void k_legendre(int nmax, int nlat, const double* __restrict__ mu,
                           double* __restrict__ P, double* __restrict__ H) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y;
  if (j >= nlat) return;
  const int M = nmax + 1;
  const double x = mu[j];
  const double s = sqrt(1.0 - x * x);
  auto eps = [m](int n) -> double {
    if (n <= m) return 0.0;
    const double nn = n;
    return sqrt((nn * nn - double(m) * m) / (4.0 * nn * nn - 1.0));
  };
  double pmm = 1.0;
  for (int k = 1; k <= m; ++k) pmm = pmm * sqrt((2.0 * k + 1.0) / (2.0 * k)) * s;
  // P rows n = m .. nmax+1 (the extra degree feeds H)
  double pm1 = 0.0, p0 = pmm;              // p(n-1), p(n)
  double* Prow = P + ((size_t)m * M) * nlat + j;
  double* Hrow = H + ((size_t)m * M) * nlat + j;
  for (int n = 0; n < m; ++n) {
    Prow[(size_t)n * nlat] = 0.0;
    Hrow[(size_t)n * nlat] = 0.0;
  }
  double pnext = pmm * sqrt(2.0 * m + 3.0) * x;  // P_{m+1}^m
  for (int n = m; n <= nmax; ++n) {
    // here p0 = P_n, pnext = P_{n+1}, pm1 = P_{n-1}
    Prow[(size_t)n * nlat] = p0;
    double h = -n * eps(n + 1) * pnext;
    if (n - 1 >= m) h = h + (n + 1.0) * eps(n) * pm1;
    Hrow[(size_t)n * nlat] = h;
    double pn2 = (pnext * x - p0 * eps(n + 1)) / eps(n + 2);  // P_{n+2}
    pm1 = p0;
    p0 = pnext;
    pnext = pn2;
  }
}

__global__ void k_twiddles(int nlon, double* tw) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nlon) return;
  double sv, cv;
  sincospi(2.0 * p / nlon, &sv, &cv);
  tw[2 * p] = cv;
  tw[2 * p + 1] = -sv;
}

__global__ void k_gw_matrices(int M, int K, double dt, const double* __restrict__ lap,
                              const double* __restrict__ ktt, const double* __restrict__ kd,
                              const double* __restrict__ whmtx,
                              const double* __restrict__ gcmtx, double* __restrict__ out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * K * K) return;
  const int l = idx % K, k = (idx / K) % K, n = idx / (K * K);
  const double dt2 = 2.0 * dt;
  const double ft = 1.0 + dt2 * ktt[n * K + k];
  const double fd = 1.0 + dt2 * kd[n * K + k];
  const double core = whmtx[k * K + l] + gcmtx[k * K + l] * ft;
  double v = -dt * dt * lap[n] * core;
  if (k == l) v += fd * ft;
  out[idx] = v;
}

// Gauss-Jordan with partial pivoting, one block per matrix, thread per row.
__global__ void k_gauss_jordan(int n, const double* __restrict__ a, double* __restrict__ ainv,
                               int* __restrict__ info) {
  extern __shared__ double sm[];
  double* A = sm;                 // [n][2n]
  __shared__ int piv;
  const int b = blockIdx.x;
  const int r = threadIdx.x;
  const int w = 2 * n;
  const double* src = a + (size_t)b * n * n;
  for (int idx = r; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx % n;
    A[i * w + j] = src[idx];
    A[i * w + n + j] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  int bad = 0;
  for (int c = 0; c < n; ++c) {
    if (r == 0) {
      int best = c;
      double bv = fabs(A[c * w + c]);
      for (int i = c + 1; i < n; ++i) {
        const double v = fabs(A[i * w + c]);
        if (v > bv) { bv = v; best = i; }
      }
      piv = (bv > 0.0) ? best : -1;
    }
    __syncthreads();
    const int p = piv;
    if (p < 0) { bad = c + 1; break; }
    if (p != c) {
      for (int j = r; j < w; j += blockDim.x) {
        const double t = A[c * w + j];
        A[c * w + j] = A[p * w + j];
        A[p * w + j] = t;
      }
    }
    __syncthreads();
    const double inv = 1.0 / A[c * w + c];
    __syncthreads();
    for (int j = r; j < w; j += blockDim.x) A[c * w + j] *= inv;
    __syncthreads();
    for (int i = r; i < n; i += blockDim.x) {
      if (i == c) continue;
      const double f = A[i * w + c];
      if (f != 0.0)
        for (int j = 0; j < w; ++j) A[i * w + j] -= f * A[c * w + j];
    }
    __syncthreads();
  }
  if (r == 0) info[b] = bad;
  double* dst = ainv + (size_t)b * n * n;
  for (int idx = r; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx % n;
    dst[idx] = bad ? 0.0 : A[i * w + n + j];
  }
}

}  // namespace lbm

using namespace lbm;

extern "C" {

const char* lbm_version(void) { return "lbm_gb300 0.1.0 (sm_103a)"; }

int lbm_gauss_legendre(int nlat, double* mu, double* gw, void* stream) {
  if (nlat < 2 || nlat > 1024 || !mu || !gw) return LBM_ERR_ARG;
  k_gauss_legendre<<<1, 512, sizeof(double), (cudaStream_t)stream>>>(nlat, mu, gw);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

int lbm_legendre_tables(int nmax, int nlat, const double* mu, double* pnm, double* hnm,
                        void* stream) {
  if (nmax < 1 || nlat < 2 || !mu || !pnm || !hnm) return LBM_ERR_ARG;
  dim3 grid((nlat + 63) / 64, nmax + 1);
  k_legendre<<<grid, 64, 0, (cudaStream_t)stream>>>(nmax, nlat, mu, pnm, hnm);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

int lbm_fft_twiddles(int nlon, double* tw, void* stream) {
  if (nlon < 2 || !tw) return LBM_ERR_ARG;
  k_twiddles<<<(nlon + 127) / 128, 128, 0, (cudaStream_t)stream>>>(nlon, tw);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

int lbm_gravity_wave_matrices(int nmax, int kmax, double dt, const double* lap,
                              const double* ktt, const double* kd, const double* whmtx,
                              const double* gcmtx, double* mats, void* stream) {
  if (nmax < 1 || kmax < 1 || !lap || !ktt || !kd || !whmtx || !gcmtx || !mats)
    return LBM_ERR_ARG;
  const int total = (nmax + 1) * kmax * kmax;
  k_gw_matrices<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      nmax + 1, kmax, dt, lap, ktt, kd, whmtx, gcmtx, mats);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

int lbm_batched_inverse(int batch, int n, const double* a, double* ainv, int* info,
                        void* stream) {
  if (batch < 1 || n < 1 || n > 64 || !a || !ainv || !info) return LBM_ERR_ARG;
  const size_t smem = (size_t)n * 2 * n * sizeof(double);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_gauss_jordan, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
  k_gauss_jordan<<<batch, 64, smem, (cudaStream_t)stream>>>(n, a, ainv, info);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

}  // extern "C"
