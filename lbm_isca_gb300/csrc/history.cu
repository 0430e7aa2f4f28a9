// Daily history accumulation on the device (model.py:257-277).
//
// The reference averages, over each output day, the trapezoid
// 0.5 (top(s) + top(s-1)) of its top-of-step diagnostics.  Every history
// field is linear in the model state (psi, chi, u, v, T, z from the spectral
// state, omega from the state and the grid ps'), so the stepper accumulates
// its spectral state and grid ps' with the same weights and forms the fields
// once per day from the mean.  This kernel is the elementwise part:
//   mode 0:  prev = cur                            (start-up call: no sample)
//   mode 1:  acc += w (cur + prev);  prev = cur    (trapezoid, w = 1/2)
// over n reals of the working precision, accumulating in FP64.
#include "lbm_gb300.h"
#include "lbm_common.cuh"

namespace lbm {

template <typename R>
__global__ void k_history(int64_t n, const R* __restrict__ cur, R* __restrict__ prev,
                          double* __restrict__ acc, double w, int mode) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const R c = cur[i];
    if (mode == 1) acc[i] += w * ((double)c + (double)prev[i]);
    prev[i] = c;
  }
}

template <typename R>
int history(int64_t n, const void* cur, void* prev, double* acc, double w, int mode,
            cudaStream_t st) {
  if (n == 0) return LBM_OK;
  const int64_t blocks64 = (n + 255) / 256;
  const int blocks = (int)(blocks64 < 152 * 16 ? blocks64 : 152 * 16);
  k_history<R><<<blocks, 256, 0, st>>>(n, (const R*)cur, (R*)prev, acc, w, mode);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}

}  // namespace lbm

extern "C" int lbm_history_accumulate(int prec, int64_t n, const void* cur, void* prev,
                                      double* acc, double w, int mode, void* stream) {
  if (n < 0 || (mode != 0 && mode != 1) || (prec != LBM_F64 && prec != LBM_F32))
    return LBM_ERR_ARG;
  if (n > 0 && (!cur || !prev || (mode == 1 && !acc))) return LBM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  return prec == LBM_F64 ? lbm::history<double>(n, cur, prev, acc, w, mode, st)
                         : lbm::history<float>(n, cur, prev, acc, w, mode, st);
}
