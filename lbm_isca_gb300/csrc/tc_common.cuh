// Blackwell (sm_103a) building blocks of the tensor-core kernels: mbarriers
// with bounded waits, bulk (TMA) copies into shared memory, tensor-memory
// (TMEM) allocation, tcgen05.mma with shared-memory operand descriptors,
// tcgen05.ld of the accumulators, and the three-way bfloat16 split of FP32
// values.  All in inline PTX; no library code.
//
// Operand layout ("K-major, no swizzle"): an operand tile of R rows (the M or
// N index) by 16 bf16 values along K is stored as 8-row x 16-byte core
// matrices; the byte offset of element (r, kk) is
//     (r / 8) * TC_SBO + (kk / 8) * TC_LBO + (r % 8) * 16 + (kk % 8) * 2
// with TC_LBO = 128 (the next 8 values along K) and TC_SBO = 256 (the next
// 8 rows).  A tile of R rows takes R * 32 bytes.
#pragma once
#include <cuda_bf16.h>
#include "lbm_common.cuh"

namespace lbm {
namespace tc {

constexpr unsigned TC_LBO = 128;
constexpr unsigned TC_SBO = 256;

LBM_D unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

LBM_HD unsigned tile_offset(int r, int kk) {
  return (unsigned)((r >> 3) * TC_SBO + (kk >> 3) * TC_LBO + (r & 7) * 16 + (kk & 7) * 2);
}

// ---- mbarriers ------------------------------------------------------------------
LBM_D void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
// Make barrier initialisations visible to the async proxy (bulk copies and
// tcgen05.commit arrive on them).
LBM_D void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
LBM_D void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
LBM_D void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}
// One poll.  A thread whose phase is not complete yet is suspended until it
// completes or about TC_SUSPEND_NS pass (a hint), so waiting warps do not
// spin on the issue slots the working warps need.
constexpr unsigned TC_SUSPEND_NS = 1000000u;
LBM_D bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(TC_SUSPEND_NS)
      : "memory");
  return ok != 0;
}
LBM_D unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;\n" : "=l"(t));
  return t;
}
// Wait for the phase of parity `parity` to complete.  Gives up after
// TC_WAIT_NS of global time: sets bit `code` of *err and returns false, so
// that no wait can hang the kernel.
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;
LBM_D bool mbar_wait(unsigned bar, unsigned parity, int* err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer_ns() - t0 > TC_WAIT_NS) break;
  }
  if (err) atomicOr(err, code);
  return false;
}

// The same wait made by a whole (converged) warp, with a warp-uniform result:
// every lane polls, the warp leaves together, lane 0 keeps the clock.
LBM_D bool warp_wait(unsigned bar, unsigned parity, int* err, int code) {
  if (__all_sync(0xffffffffu, mbar_try_wait(bar, parity))) return true;
  const unsigned long long t0 = globaltimer_ns();
  for (;;) {
    if (__all_sync(0xffffffffu, mbar_try_wait(bar, parity))) return true;
    const int late = globaltimer_ns() - t0 > TC_WAIT_NS ? 1 : 0;
    if (__shfl_sync(0xffffffffu, late, 0)) break;
  }
  if ((threadIdx.x & 31) == 0 && err) atomicOr(err, code);
  return false;
}

// Writes of the generic proxy (st.shared) made visible to the async proxy
// (bulk copies, tcgen05.mma operand reads).
LBM_D void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// ---- bulk copies (TMA engine) --------------------------------------------------
// `bytes` from global `src` to shared `dst`, both 16-byte aligned, bytes a
// multiple of 16; completion counted on mbarrier `bar` (expect_tx first).
LBM_D void bulk_g2s(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
      ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// ---- tensor memory -----------------------------------------------------------------
// Called by one whole warp; the base address is written to shared `slot`.
LBM_D void tmem_alloc(unsigned slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
LBM_D void tmem_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols)
               : "memory");
}
LBM_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
LBM_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// ---- descriptors -------------------------------------------------------------------
// Shared-memory matrix descriptor of a K-major, unswizzled operand tile.
LBM_D uint64_t smem_desc(unsigned addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(TC_LBO >> 4) << 16) |
         ((uint64_t)(TC_SBO >> 4) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16 with bf16 A and B (both K-major), FP32
// accumulator, M x N.
LBM_HD unsigned idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) |
         ((unsigned)(M >> 4) << 24);
}

// D (TMEM) (+)= A (smem) * B (smem)^T, one M x N x 16 step; issued by one thread.
LBM_D void mma_bf16(unsigned d_tmem, uint64_t adesc, uint64_t bdesc, unsigned idesc,
                    bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((unsigned)accumulate)
      : "memory");
}
// Arrive once on `bar` when every tcgen05 operation this thread issued so far
// has completed.
LBM_D void mma_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::
                   "r"(bar)
               : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes
// 32 (w % 4) .. + 31; taddr carries the lane base in its upper 16 bits).
LBM_D void tmem_ld16(unsigned taddr, float* v) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- three-way bfloat16 split ----------------------------------------------------
// x = b0 + b1 + b2 to about 24 bits: b0 = bf16(x), b1 = bf16(x - b0),
// b2 = bf16(x - b0 - b1); each difference is exact in FP32.  The products
// kept by the split contractions are b0 c0 + b0 c1 + b1 c0 + b0 c2 + b1 c1 +
// b2 c0 (every term down to the third order; the dropped ones are below
// 2^-24 of the product).
struct Split3 { __nv_bfloat16 p[3]; };
LBM_D Split3 split3(float x) {
  Split3 s;
  s.p[0] = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(s.p[0]);
  s.p[1] = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(s.p[1]);
  s.p[2] = __float2bfloat16_rn(r2);
  return s;
}
// The same split of two values at once (packed conversions): w[p] holds
// piece p of a in its low and of b in its high 16 bits.
LBM_D void split3_pair(float a, float b, unsigned* w) {
  const __nv_bfloat162 h0 = __floats2bfloat162_rn(a, b);
  const float2 f0 = __bfloat1622float2(h0);
  const float ra = a - f0.x, rb = b - f0.y;
  const __nv_bfloat162 h1 = __floats2bfloat162_rn(ra, rb);
  const float2 f1 = __bfloat1622float2(h1);
  const __nv_bfloat162 h2 = __floats2bfloat162_rn(ra - f1.x, rb - f1.y);
  w[0] = *reinterpret_cast<const unsigned*>(&h0);
  w[1] = *reinterpret_cast<const unsigned*>(&h1);
  w[2] = *reinterpret_cast<const unsigned*>(&h2);
}
// Eight values along K -> three 16-byte rows (one per piece) of a tile.
LBM_D void split3_store8(const float* x, unsigned char* row0, unsigned char* row1,
                         unsigned char* row2) {
  unsigned u[3][4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    unsigned w[3];
    split3_pair(x[2 * q], x[2 * q + 1], w);
#pragma unroll
    for (int p = 0; p < 3; ++p) u[p][q] = w[p];
  }
  *reinterpret_cast<uint4*>(row0) = make_uint4(u[0][0], u[0][1], u[0][2], u[0][3]);
  *reinterpret_cast<uint4*>(row1) = make_uint4(u[1][0], u[1][1], u[1][2], u[1][3]);
  *reinterpret_cast<uint4*>(row2) = make_uint4(u[2][0], u[2][1], u[2][2], u[2][3]);
}

}  // namespace tc
}  // namespace lbm
