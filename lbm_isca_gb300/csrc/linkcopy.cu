// Copies between device memory and pinned host memory carried out by SM
// loads and stores over the CPU-GPU link (NVLink-C2C on a Grace-Blackwell
// node) rather than by a copy engine: the path by which the model's inputs
// (heatings) reach the GPU and its results (the grid state) come back.
#include "lbm_common.cuh"

namespace lbm {

__global__ void __launch_bounds__(256) k_link_copy(const uint4* __restrict__ src,
                                                   uint4* __restrict__ dst, size_t n16,
                                                   const unsigned char* __restrict__ src_tail,
                                                   unsigned char* __restrict__ dst_tail,
                                                   int tail) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  // four independent 16-byte transfers in flight per thread
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride],
                d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n16; i += stride) dst[i] = src[i];
  if (blockIdx.x == 0 && (int)threadIdx.x < tail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

static bool device_accessible(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged ||
         (a.type == cudaMemoryTypeHost && a.devicePointer == p);
}

}  // namespace lbm

using namespace lbm;

extern "C" int lbm_link_copy(void* dst, const void* src, int64_t bytes, void* stream) {
  if (bytes < 0 || (bytes > 0 && (!dst || !src))) return LBM_ERR_ARG;
  if (bytes == 0) return LBM_OK;
  if (((uintptr_t)dst & 15) || ((uintptr_t)src & 15)) return LBM_ERR_ARG;
  if (!device_accessible(dst) || !device_accessible(src)) return LBM_ERR_ARG;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t n16 = (size_t)bytes / 16;
  const int tail = (int)(bytes - (int64_t)n16 * 16);
  size_t blocks = (n16 + 255) / 256;
  const size_t cap = (size_t)(sms > 0 ? sms : 1) * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  k_link_copy<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      (const uint4*)src, (uint4*)dst, n16, (const unsigned char*)src + n16 * 16,
      (unsigned char*)dst + n16 * 16, tail);
  LBM_LAUNCH_CHECK();
  return LBM_OK;
}
