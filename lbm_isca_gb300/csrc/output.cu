// GrADS history records of one output day, packed on the device.
//
// The history writer of the reference (output.py:46-71) emits, per day, one
// Fortran sequential record per level of psi, chi, u, v, w, t, z and one of
// ps: a big-endian int32 byte count, the field's npts values as big-endian
// real*4, the byte count again.  z first gets the surface-pressure term
// (ps * zmul) / zdiv, evaluated in that order (output.py:64-65).  One thread
// per output word.

#include "lbm_common.cuh"

namespace lbm {

struct GradsFields {
  const double* f[8];   // psi chi u v w t z ([npts][kmax]), ps ([npts])
};

__global__ void k_grads_records(GradsFields g, long long npts, int kmax, int apply_z,
                                double zmul, double zdiv, unsigned* __restrict__ out,
                                long long nwords) {
  const long long rl = npts + 2;                        // words per record
  const unsigned marker = __byte_perm((unsigned)(4 * npts), 0, 0x0123);
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nwords;
       w += (long long)gridDim.x * blockDim.x) {
    const long long rec = w / rl, pos = w - rec * rl;
    unsigned word;
    if (pos == 0 || pos == rl - 1) {
      word = marker;
    } else {
      const long long i = pos - 1;
      double v;
      if (rec < 7LL * kmax) {
        const int fld = (int)(rec / kmax), k = (int)(rec - (long long)fld * kmax);
        v = g.f[fld][i * kmax + k];
        if (fld == 6 && apply_z) v += (g.f[7][i] * zmul) / zdiv;
      } else {
        v = g.f[7][i];
      }
      word = __byte_perm(__float_as_uint(__double2float_rn(v)), 0, 0x0123);
    }
    out[w] = word;
  }
}

}  // namespace lbm

using namespace lbm;

extern "C" int lbm_grads_records(int64_t npts, int kmax, const double* const* fields,
                                 int apply_z, double zmul, double zdiv, uint32_t* out,
                                 void* stream) {
  if (npts < 1 || kmax < 1 || !fields || !out || 4 * npts > 0x7fffffffLL || zdiv == 0.0)
    return LBM_ERR_ARG;
  GradsFields g;
  for (int i = 0; i < 8; ++i) {
    if (!fields[i]) return LBM_ERR_ARG;
    g.f[i] = fields[i];
  }
  const long long nwords = (7LL * kmax + 1) * (npts + 2);
  const int nt = 256;
  long long nb = (nwords + nt - 1) / nt;
  if (nb > 4096) nb = 4096;
  k_grads_records<<<(unsigned)nb, nt, 0, (cudaStream_t)stream>>>(g, npts, kmax, apply_z, zmul,
                                                                   zdiv, out, nwords);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}
