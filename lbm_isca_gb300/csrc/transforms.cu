// Spectral transforms on the reference array layouts: the building blocks of
// Spectral.grid_to_wave / wave_to_grid / hgrad / uv_to_vordiv / psichi_to_uv
// (spectral.py:159-276).  The fused ensemble stepper has its own kernels;
// these serve the drop-in Python API, setup and diagnostics.
#include "lbm_common.cuh"
#include "lbm_fft.cuh"

namespace lbm {

constexpr int FT_THREADS = 256;   // threads per block of the Fourier kernels
constexpr int FT_COLS = 32;       // columns (levels) per block

// grid[b][j][i][c] -> four[b][m][j][c] = jscale[j]/I rfft.  Block = (j, b,
// column chunk); the chunk's I x CC slab is staged transposed in shared
// memory, teams of R1 threads transform one column each.
template <typename R, int I>
__global__ void __launch_bounds__(FT_THREADS)
k_fourier_fwd(int J, int C, int M, const R* __restrict__ grid, const R* __restrict__ jscale,
              const C2<R>* __restrict__ twg, C2<R>* __restrict__ four) {
  constexpr int R1 = FftShape<I>::R1;
  constexpr int NTEAM = FT_THREADS / R1;
  constexpr int SCR = fft_team_scratch<I>();
  extern __shared__ unsigned char smraw[];
  C2<R>* tw = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* scr = tw + I;                       // [NTEAM][SCR]
  C2<R>* outst = scr + NTEAM * SCR;          // [M][FT_COLS]
  R* slab = reinterpret_cast<R*>(outst + M * FT_COLS);  // [FT_COLS][I+1]
  const int j = blockIdx.x, b = blockIdx.y, c0 = blockIdx.z * FT_COLS;
  const int cc = min(FT_COLS, C - c0);
  const int tid = threadIdx.x;
  for (int p = tid; p < I; p += FT_THREADS) tw[p] = twg[p];
  const R* src = grid + ((size_t)b * J + j) * I * C;
  for (int idx = tid; idx < I * cc; idx += FT_THREADS) {
    const int i = idx / cc, c = idx % cc;
    slab[c * (I + 1) + i] = src[(size_t)i * C + c0 + c];
  }
  __syncthreads();
  const R scale = (jscale ? jscale[j] : R(1)) / R(I);
  const int team = tid / R1, t = tid % R1;
  for (int c = team; c < cc; c += NTEAM) {
    team_rfft_fwd<I>(t, slab + c * (I + 1), 1, scr + team * SCR, tw, M, scale,
                     [&](int m, C2<R> X) { outst[m * FT_COLS + c] = X; });
  }
  __syncthreads();
  for (int idx = tid; idx < M * cc; idx += FT_THREADS) {
    const int m = idx / cc, c = idx % cc;
    four[(((size_t)b * M + m) * J + j) * C + c0 + c] = outst[m * FT_COLS + c];
  }
}

template <typename R, int I>
__global__ void __launch_bounds__(FT_THREADS)
k_fourier_inv(int J, int C, int M, const C2<R>* __restrict__ four, const R* __restrict__ jscale,
              const C2<R>* __restrict__ twg, R* __restrict__ grid) {
  constexpr int R1 = FftShape<I>::R1;
  constexpr int NTEAM = FT_THREADS / R1;
  constexpr int SCR = fft_team_scratch<I>();
  extern __shared__ unsigned char smraw[];
  C2<R>* tw = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* scr = tw + I;
  C2<R>* inst = scr + NTEAM * SCR;           // [FT_COLS][M]
  R* slab = reinterpret_cast<R*>(inst + M * FT_COLS);  // [FT_COLS][I+1]
  const int j = blockIdx.x, b = blockIdx.y, c0 = blockIdx.z * FT_COLS;
  const int cc = min(FT_COLS, C - c0);
  const int tid = threadIdx.x;
  for (int p = tid; p < I; p += FT_THREADS) tw[p] = twg[p];
  for (int idx = tid; idx < M * cc; idx += FT_THREADS) {
    const int m = idx / cc, c = idx % cc;
    inst[c * M + m] = four[(((size_t)b * M + m) * J + j) * C + c0 + c];
  }
  __syncthreads();
  const R scale = jscale ? jscale[j] : R(1);
  const int team = tid / R1, t = tid % R1;
  for (int c = team; c < cc; c += NTEAM) {
    const C2<R>* X = inst + c * M;
    team_rfft_inv<I>(t, [&](int m) { return X[m]; }, M, scr + team * SCR, tw,
                     slab + c * (I + 1), 1, scale);
  }
  __syncthreads();
  R* dst = grid + ((size_t)b * J + j) * I * C;
  for (int idx = tid; idx < I * cc; idx += FT_THREADS) {
    const int i = idx / cc, c = idx % cc;
    dst[(size_t)i * C + c0 + c] = slab[c * (I + 1) + i];
  }
}

constexpr int LG_COLS = 16;     // columns per block of the Legendre kernels
constexpr int LG_ROWS = 16;     // thread rows (n or j)

// spec[b][m][n][c] (+)= nfac[n] (ca sum_j ta f_a + sb cb sum_j tb f_b)
template <typename R>
__global__ void __launch_bounds__(LG_COLS * LG_ROWS)
k_leg_anal(int M, int J, int C, const C2<R>* __restrict__ fa, const R* __restrict__ ta,
           int ima, const C2<R>* __restrict__ fb, const R* __restrict__ tb, int imb, R sb,
           const R* __restrict__ nfac, int accumulate, C2<R>* __restrict__ spec) {
  extern __shared__ unsigned char smraw[];
  C2<R>* sa = reinterpret_cast<C2<R>*>(smraw);   // [J][LG_COLS]
  C2<R>* sbb = sa + J * LG_COLS;
  const int m = blockIdx.x, b = blockIdx.y, c0 = blockIdx.z * LG_COLS;
  const int cc = min(LG_COLS, C - c0);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * LG_COLS + tx;
  for (int idx = tid; idx < J * LG_COLS; idx += LG_COLS * LG_ROWS) {
    const int jj = idx / LG_COLS, c = idx % LG_COLS;
    const size_t g = (((size_t)b * M + m) * J + jj) * C + c0 + c;
    sa[idx] = (c < cc) ? fa[g] : cmk<R>(0, 0);
    if (fb) sbb[idx] = (c < cc) ? fb[g] : cmk<R>(0, 0);
  }
  __syncthreads();
  if (tx >= cc) return;
  const R mm = R(m);
  for (int n = ty; n < M; n += LG_ROWS) {
    const size_t o = (((size_t)b * M + m) * M + n) * C + c0 + tx;
    if (n < m) {
      if (!accumulate) spec[o] = cmk<R>(0, 0);
      continue;
    }
    const R* pa = ta + ((size_t)m * M + n) * J;
    C2<R> acc = cmk<R>(0, 0), accb = cmk<R>(0, 0);
    for (int jj = 0; jj < J; ++jj) cfma(acc, pa[jj], sa[jj * LG_COLS + tx]);
    if (ima) acc = im_mul(acc, mm);
    if (fb) {
      const R* pb = tb + ((size_t)m * M + n) * J;
      for (int jj = 0; jj < J; ++jj) cfma(accb, pb[jj], sbb[jj * LG_COLS + tx]);
      if (imb) accb = im_mul(accb, mm);
      acc = acc + accb * sb;
    }
    if (nfac) acc = acc * nfac[n];
    if (accumulate) acc = acc + spec[o];
    spec[o] = acc;
  }
}

// four[b][m][j][c] = sum_n ta[m][n][j] ca na[n] sa + sb sum_n tb cb nb[n] sb_
template <typename R>
__global__ void __launch_bounds__(LG_COLS * LG_ROWS)
k_leg_synth(int M, int J, int C, const C2<R>* __restrict__ sa, const R* __restrict__ ta,
            int ima, const R* __restrict__ na, const C2<R>* __restrict__ sbp,
            const R* __restrict__ tb, int imb, const R* __restrict__ nb, R sb,
            C2<R>* __restrict__ four) {
  extern __shared__ unsigned char smraw[];
  C2<R>* xa = reinterpret_cast<C2<R>*>(smraw);   // [M][LG_COLS]
  C2<R>* xb = xa + M * LG_COLS;
  const int m = blockIdx.x, b = blockIdx.y, c0 = blockIdx.z * LG_COLS;
  const int cc = min(LG_COLS, C - c0);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * LG_COLS + tx;
  const R mm = R(m);
  for (int idx = tid; idx < M * LG_COLS; idx += LG_COLS * LG_ROWS) {
    const int n = idx / LG_COLS, c = idx % LG_COLS;
    C2<R> va = cmk<R>(0, 0), vb = cmk<R>(0, 0);
    if (c < cc && n >= m) {
      const size_t g = (((size_t)b * M + m) * M + n) * C + c0 + c;
      va = sa[g];
      if (ima) va = im_mul(va, mm);
      if (na) va = va * na[n];
      if (sbp) {
        vb = sbp[g];
        if (imb) vb = im_mul(vb, mm);
        if (nb) vb = vb * nb[n];
        vb = vb * sb;
      }
    }
    xa[idx] = va;
    xb[idx] = vb;
  }
  __syncthreads();
  if (tx >= cc) return;
  for (int jj = ty; jj < J; jj += LG_ROWS) {
    C2<R> acc = cmk<R>(0, 0);
    for (int n = m; n < M; ++n) {
      cfma(acc, ta[((size_t)m * M + n) * J + jj], xa[n * LG_COLS + tx]);
      if (sbp) cfma(acc, tb[((size_t)m * M + n) * J + jj], xb[n * LG_COLS + tx]);
    }
    four[(((size_t)b * M + m) * J + jj) * C + c0 + tx] = acc;
  }
}

template <typename R, int I>
int launch_fourier(bool fwd, int B, int J, int C, int M, const void* in, const void* js,
                   const void* tw, void* out, cudaStream_t st) {
  constexpr int R1 = FftShape<I>::R1;
  constexpr int NTEAM = FT_THREADS / R1;
  const size_t smem = sizeof(C2<R>) * (I + NTEAM * fft_team_scratch<I>() + M * FT_COLS) +
                      sizeof(R) * FT_COLS * (I + 1);
  dim3 grid(J, B, (C + FT_COLS - 1) / FT_COLS);
  if (fwd) {
    cudaFuncSetAttribute(k_fourier_fwd<R, I>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    k_fourier_fwd<R, I><<<grid, FT_THREADS, smem, st>>>(
        J, C, M, (const R*)in, (const R*)js, (const C2<R>*)tw, (C2<R>*)out);
  } else {
    cudaFuncSetAttribute(k_fourier_inv<R, I>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    k_fourier_inv<R, I><<<grid, FT_THREADS, smem, st>>>(
        J, C, M, (const C2<R>*)in, (const R*)js, (const C2<R>*)tw, (R*)out);
  }
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

template <typename R>
int fourier_dispatch(bool fwd, int B, int J, int I, int C, int nmax, const void* in,
                     const void* js, const void* tw, void* out, cudaStream_t st) {
  const int M = nmax + 1;
  if (B < 1 || J < 2 || C < 1 || M < 1 || 2 * M > I || !in || !tw || !out) return LBM_ERR_ARG;
  switch (I) {
    case 64: return launch_fourier<R, 64>(fwd, B, J, C, M, in, js, tw, out, st);
    case 128: return launch_fourier<R, 128>(fwd, B, J, C, M, in, js, tw, out, st);
    case 256: return launch_fourier<R, 256>(fwd, B, J, C, M, in, js, tw, out, st);
    default: return LBM_ERR_ARG;
  }
}

template <typename R>
static int leg_anal(int B, int nmax, int J, int C, const void* fa, const void* ta, int ima,
                    const void* fb, const void* tb, int imb, double sb, const void* nfac,
                    int acc, void* spec, cudaStream_t st) {
  const int M = nmax + 1;
  if (B < 1 || M < 1 || J < 2 || C < 1 || !fa || !ta || !spec || (fb && !tb))
    return LBM_ERR_ARG;
  const size_t smem = sizeof(C2<R>) * 2 * J * LG_COLS;
  cudaFuncSetAttribute(k_leg_anal<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid(M, B, (C + LG_COLS - 1) / LG_COLS), block(LG_COLS, LG_ROWS);
  k_leg_anal<R><<<grid, block, smem, st>>>(M, J, C, (const C2<R>*)fa, (const R*)ta, ima,
                                           (const C2<R>*)fb, (const R*)tb, imb, R(sb),
                                           (const R*)nfac, acc, (C2<R>*)spec);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

template <typename R>
static int leg_synth(int B, int nmax, int J, int C, const void* sa, const void* ta, int ima,
                     const void* na, const void* sbp, const void* tb, int imb, const void* nb,
                     double sb, void* four, cudaStream_t st) {
  const int M = nmax + 1;
  if (B < 1 || M < 1 || J < 2 || C < 1 || !sa || !ta || !four || (sbp && !tb))
    return LBM_ERR_ARG;
  const size_t smem = sizeof(C2<R>) * 2 * M * LG_COLS;
  cudaFuncSetAttribute(k_leg_synth<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid(M, B, (C + LG_COLS - 1) / LG_COLS), block(LG_COLS, LG_ROWS);
  k_leg_synth<R><<<grid, block, smem, st>>>(M, J, C, (const C2<R>*)sa, (const R*)ta, ima,
                                            (const R*)na, (const C2<R>*)sbp, (const R*)tb,
                                            imb, (const R*)nb, R(sb), (C2<R>*)four);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

}  // namespace lbm

using namespace lbm;

extern "C" {

int lbm_fourier_forward(int prec, int batch, int nlat, int nlon, int ncol, int nmax,
                        const void* grid, const void* jscale, const void* tw, void* four,
                        void* stream) {
  if (prec == LBM_F64)
    return fourier_dispatch<double>(true, batch, nlat, nlon, ncol, nmax, grid, jscale, tw,
                                    four, (cudaStream_t)stream);
  if (prec == LBM_F32)
    return fourier_dispatch<float>(true, batch, nlat, nlon, ncol, nmax, grid, jscale, tw, four,
                                   (cudaStream_t)stream);
  return LBM_ERR_ARG;
}

int lbm_fourier_inverse(int prec, int batch, int nlat, int nlon, int ncol, int nmax,
                        const void* four, const void* jscale, const void* tw, void* grid,
                        void* stream) {
  if (prec == LBM_F64)
    return fourier_dispatch<double>(false, batch, nlat, nlon, ncol, nmax, four, jscale, tw,
                                    grid, (cudaStream_t)stream);
  if (prec == LBM_F32)
    return fourier_dispatch<float>(false, batch, nlat, nlon, ncol, nmax, four, jscale, tw,
                                   grid, (cudaStream_t)stream);
  return LBM_ERR_ARG;
}

int lbm_legendre_analysis(int prec, int batch, int nmax, int nlat, int ncol, const void* fa,
                          const void* ta, int ima, const void* fb, const void* tb, int imb,
                          double sb, const void* nfac, int accumulate, void* spec,
                          void* stream) {
  if (prec == LBM_F64)
    return leg_anal<double>(batch, nmax, nlat, ncol, fa, ta, ima, fb, tb, imb, sb, nfac,
                            accumulate, spec, (cudaStream_t)stream);
  if (prec == LBM_F32)
    return leg_anal<float>(batch, nmax, nlat, ncol, fa, ta, ima, fb, tb, imb, sb, nfac,
                           accumulate, spec, (cudaStream_t)stream);
  return LBM_ERR_ARG;
}

int lbm_legendre_synthesis(int prec, int batch, int nmax, int nlat, int ncol, const void* sa,
                           const void* ta, int ima, const void* na, const void* sb_,
                           const void* tb, int imb, const void* nb, double sb, void* four,
                           void* stream) {
  if (prec == LBM_F64)
    return leg_synth<double>(batch, nmax, nlat, ncol, sa, ta, ima, na, sb_, tb, imb, nb, sb,
                             four, (cudaStream_t)stream);
  if (prec == LBM_F32)
    return leg_synth<float>(batch, nmax, nlat, ncol, sa, ta, ima, na, sb_, tb, imb, nb, sb,
                            four, (cudaStream_t)stream);
  return LBM_ERR_ARG;
}

}  // extern "C"
