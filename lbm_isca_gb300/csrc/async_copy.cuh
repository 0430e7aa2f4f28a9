// Asynchronous global -> shared copies (cp.async) with completion groups.
#pragma once
#include "lbm_common.cuh"

namespace lbm {

// 16 bytes; both addresses 16-byte aligned.
LBM_D void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
// One complex value of the working precision (8 or 16 bytes).
template <typename R> LBM_D void cp_async_c2(C2<R>* smem, const C2<R>* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(C2<R>) == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
LBM_D void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// Wait until at most N of this thread's groups are still in flight.
template <int N> LBM_D void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Bulk prefetch of `bytes` (a multiple of 16) at `gmem` (16-byte aligned)
// into L2; no completion is tracked.
LBM_D void prefetch_l2_bulk(const void* gmem, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(gmem), "r"(bytes) : "memory");
}

}  // namespace lbm
