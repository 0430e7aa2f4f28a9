// Longitude analysis of the FP32 stepper (k_fdft's work: grid9 -> af, afs):
// the 9K level rows on the tensor cores (k_fdft_tc: bfloat16 split operands,
// FP32 accumulation in TMEM), the two surface rows on the FMA pipes
// (k_fdft_surf).
//
// Per (member, latitude) unit the weighted Fourier coefficients of the R =
// 9K level rows are one product
//   D[L][n] = sum_i W[L][i] G[n][i],  L = 2m + c,
// with W[2m][i] = cos(2 pi m i / I) / I and W[2m+1][i] = -sin(2 pi m i / I) /
// I (so D[2m] + i D[2m+1] is the rfft coefficient of row n over I, as
// Spectral._fft_fwd forms it, spectral.py:159-164), K = longitudes in steps
// of 16, N = the unit's rows (R rounded up to 16, at most 256).  The table W
// (128 lanes, split from FP64 into three bf16 pieces) stays in shared memory
// for the whole kernel; the grid rows are split in registers from FP32
// loads (the next unit pulled into L2 ahead) into a four-slot ring.  The
// epilogue combines a level's rows as k_fdft does -- a3 = wg X(gt) -
// wd i m X(xu), a5 = wg X(g) - wd i m X(yu), wd X(fu), wd X(fv), wg X(ke),
// wd X(xv), wd X(yv) -- with the i m terms taken from the partner lane
// (L ^ 1), stages the unit's af rows in shared memory and writes them as
// contiguous runs.
//
// Why the surface rows stay on FMA: the tensor cores' FP32 accumulation
// rounds toward zero, so every coefficient comes out smaller in magnitude by
// about 2.6e-7 relative (measured on GB300, T42: the FMA kernel's signed
// error is 1e-9).  For tendencies that is noise, but the second surface row
// is pi(t - dt), which goes spectral -> grid -> spectral every step (its
// Robert-Asselin filter runs in grid space): the shrink would compound step
// after step (the bf16x3 run then drifts to 4e-5 in pi at day 30).  The
// Legendre tensor-core kernels keep the surface fields on FMA for the same
// reason.
//
// Roles of k_fdft_tc (one persistent CTA per SM): warp 0 loads the table
// image once and prefetches units into L2; warp 1 TMEM and MMA issue; warps
// 2..13 split the grid rows; warps 14..21 the epilogue (each TMEM lane
// quarter read by two warps, one per half of the levels).  Bounded waits as in
// legendre_tc.cuh.  Supported: nlon <= 128 (the table's 2 (nmax + 1) <= 128
// lanes), nlon a power of two, and 9 kmax <= 256 rows.
#pragma once
#include "tc_common.cuh"
#include "async_copy.cuh"

namespace lbm {

constexpr int FTC_BSLOTS = 4;
constexpr int FTC_CONV_WARPS = 12;     // 384 threads, at most two items each (2 NR <= 512)
constexpr int FTC_EPI_WARPS = 8;       // two warps per TMEM lane quarter, half the levels each
constexpr int FTC_CONV = 32 * FTC_CONV_WARPS;
constexpr int FTC_EPI = 32 * FTC_EPI_WARPS;
constexpr int FTC_THREADS = 32 * (2 + FTC_CONV_WARPS + FTC_EPI_WARPS);
static_assert(FTC_EPI == 256, "the epilogue's named barrier counts 256 threads");
static_assert(2 * FTC_CONV >= 512, "two items per conversion thread cover 2 NR <= 512");
constexpr int FTC_PREFETCH = 1;        // units of grid rows pulled into L2 ahead (swept: 0-6)

// Floats per wavenumber in the epilogue's staging area: the K x 7 complex of
// a unit's af row plus 4, so that the 16 wavenumbers of a warp's stores fall
// on 8 bank groups instead of 4 (the copy-out keeps 16-byte alignment).
LBM_HD int ftc_stage_stride(int K) { return K * 14 + 4; }

struct FtcPlan {
  int R, NR, KS, nunits, tcols;
  unsigned tab_bytes, b_bytes, out_bytes, smem;
};

LBM_HD FtcPlan ftc_plan(int E, int J, int I, int K, int N) {
  FtcPlan p;
  p.R = 9 * K;
  p.NR = (p.R + 15) / 16 * 16;
  p.KS = I / 16;
  p.nunits = E * J;
  const int cols = 2 * p.NR;
  p.tcols = cols <= 128 ? 128 : cols <= 256 ? 256 : 512;
  p.tab_bytes = (unsigned)(p.KS * 3 * 4096);            // 128 lanes x 16 x 3 pieces per step
  p.b_bytes = (unsigned)(3 * p.NR * 32);
  p.out_bytes = (unsigned)((N + 1) * ftc_stage_stride(K) * 4);
  p.smem = 2048 + p.tab_bytes + FTC_BSLOTS * ((p.b_bytes + 1023) / 1024 * 1024) +
           (p.out_bytes + 1023) / 1024 * 1024;
  return p;
}

LBM_HD bool ftc_supported(int I, int K, int N) {
  return I <= 128 && 2 * (N + 1) <= 128 && 9 * K <= 256 && (I % 16) == 0 && !(I & (I - 1));
}

struct FtcSmem {
  unsigned long long tab, bfull[FTC_BSLOTS], bempty[FTC_BSLOTS], accfull[2], accempty[2], done;
  unsigned tslot;
};

// B row of level row q (grid row 2 + q): ordered (field, level) so that a
// field's levels are adjacent columns of D.
LBM_D int ftc_brow(int q, int K) {
  const int k = q / 9, f = q - 9 * k;
  return f * K + k;
}

__global__ void __launch_bounds__(FTC_THREADS, 1)
    k_fdft_tc(SD<float> d, const unsigned char* __restrict__ tab, FtcPlan pl, int nprod) {
  extern __shared__ unsigned char smraw_ftc[];
  unsigned char* base = smraw_ftc + ((1024u - (tc::smem_addr(smraw_ftc) & 1023u)) & 1023u);
  FtcSmem* sm = reinterpret_cast<FtcSmem*>(base);
  unsigned char* stab = base + 1024;
  const unsigned bslot = (pl.b_bytes + 1023) / 1024 * 1024;
  unsigned char* bring = stab + pl.tab_bytes;
  float* stage = reinterpret_cast<float*>(bring + FTC_BSLOTS * bslot);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int J = d.J, I = d.I, K = d.K, M = d.M, KS = pl.KS, R = pl.R, NR = pl.NR;
  int* err = d.err;
  using namespace tc;

  if (threadIdx.x == 0) {
    mbar_init(smem_addr(&sm->tab), 1);
    for (int i = 0; i < FTC_BSLOTS; ++i) {
      mbar_init(smem_addr(&sm->bfull[i]), FTC_CONV_WARPS);
      mbar_init(smem_addr(&sm->bempty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_addr(&sm->accfull[i]), 1);
      mbar_init(smem_addr(&sm->accempty[i]), FTC_EPI_WARPS);
    }
    mbar_init(smem_addr(&sm->done), 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(smem_addr(&sm->tslot), (unsigned)pl.tcols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tbase = sm->tslot;
  bool ok = true;
  const float* g9 = d.grid9;
  const size_t unit_floats = (size_t)(2 + R) * I;      // a unit's grid rows, surface first

  if (warp == 0) {
    // ---------------- table once, then L2 prefetch of the units ahead ----------
    if (lane == 0) {
      const unsigned bar = smem_addr(&sm->tab);
      mbar_expect_tx(bar, pl.tab_bytes);
      for (unsigned o = 0; o < pl.tab_bytes; o += 4096u * 3u)
        bulk_g2s(smem_addr(stab + o), tab + o, 4096u * 3u, bar);
      // the copies land before the CTA winds down
      mbar_wait(bar, 0, err, ATC_ERR);
      int n = 0;
      for (int u = blockIdx.x; u < pl.nunits && n < FTC_PREFETCH; u += gridDim.x, ++n)
        prefetch_l2_bulk(g9 + (size_t)u * unit_floats, (unsigned)(unit_floats * 4));
    }
  } else if (warp == 1) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      const int q0 = nprod == 3 ? 3 : 0;
      const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
      const unsigned idesc = idesc_bf16(128, NR);
      ok = mbar_wait(smem_addr(&sm->tab), 0, err, ATC_ERR);
      unsigned a = 0, ul = 0;
      const uint64_t tdesc = smem_desc(smem_addr(stab));
      for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x, ++ul) {
        const int b = ul & 1;
        ok = mbar_wait(smem_addr(&sm->accempty[b]), ((ul >> 1) & 1u) ^ 1u, err, ATC_ERR);
        if (!ok) break;
        tc_fence_after();
        const unsigned dcol = tbase + (unsigned)(b * NR);
        bool acc = false;
        for (int s = 0; s < KS && ok; ++s, ++a) {
          const int slot = a % FTC_BSLOTS;
          ok = mbar_wait(smem_addr(&sm->bfull[slot]), (a / FTC_BSLOTS) & 1u, err, ATC_ERR);
          if (!ok) break;
          tc_fence_after();
          const uint64_t bdesc = smem_desc(smem_addr(bring + slot * bslot));
          const uint64_t ad = tdesc + (uint64_t)((s * 3u * 4096u) >> 4);
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            if (q < q0) continue;
            mma_bf16(dcol, ad + (uint64_t)((pa[q] * 4096u) >> 4),
                     bdesc + (uint64_t)((pb[q] * (unsigned)NR * 32u) >> 4), idesc, acc);
            acc = true;
          }
          mma_commit(smem_addr(&sm->bempty[slot]));
        }
        if (!ok) break;
        mma_commit(smem_addr(&sm->accfull[b]));
      }
      mma_commit(smem_addr(&sm->done));
      mbar_wait(smem_addr(&sm->done), 0, err, ATC_ERR);
    }
  } else if (warp < 2 + FTC_CONV_WARPS) {
    // ---------------- conversion: grid rows -> B tiles ----------------
    // (B row, 8-longitude chunk) items it = ct and ct + FTC_CONV per thread
    // (2 NR <= 512 items): the 8 lanes of a quarter warp take 8 consecutive B
    // rows of one chunk, so each 16-byte store of a quarter warp fills one
    // 128-byte core-matrix row group (no bank conflicts).  The next step's
    // rows are loaded into registers before this step's are split (the
    // loads' latency is hidden behind the split and the wait for a slot).
    const int ct = threadIdx.x - 64;
    int br[2], chk[2], q[2];
    bool live[2], data[2];
    unsigned off[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int it = ct + h * FTC_CONV;
      chk[h] = (it >> 3) & 1;
      br[h] = (it & 7) | ((it >> 4) << 3);       // B row (field f = br / K, level br % K)
      live[h] = it < 2 * NR;                     // padding rows past R stay zero
      data[h] = live[h] && br[h] < R;
      q[h] = 9 * (br[h] % K) + br[h] / K;        // its level row: ftc_brow(q, K) == br
      off[h] = tile_offset(br[h], chk[h] * 8);
    }
    auto load = [&](int h, int u, int s, float4& x0, float4& x1) {
      if (data[h] && u < pl.nunits) {
        const float4* src = reinterpret_cast<const float4*>(
            g9 + (size_t)u * unit_floats + (size_t)(2 + q[h]) * I + s * 16 + chk[h] * 8);
        x0 = __ldg(src);
        x1 = __ldg(src + 1);
      } else {
        x0 = x1 = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    };
    float4 n0[2], n1[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) load(h, blockIdx.x, 0, n0[h], n1[h]);
    unsigned a = 0;
    for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x) {
      if (ct == 0) {
        const int un = u + FTC_PREFETCH * gridDim.x;
        if (un < pl.nunits)
          prefetch_l2_bulk(g9 + (size_t)un * unit_floats, (unsigned)(unit_floats * 4));
      }
      for (int s = 0; s < KS && ok; ++s, ++a) {
        const int slot = a % FTC_BSLOTS;
        float x[2][8];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          x[h][0] = n0[h].x; x[h][1] = n0[h].y; x[h][2] = n0[h].z; x[h][3] = n0[h].w;
          x[h][4] = n1[h].x; x[h][5] = n1[h].y; x[h][6] = n1[h].z; x[h][7] = n1[h].w;
          if (s + 1 < KS) load(h, u, s + 1, n0[h], n1[h]);
          else load(h, u + gridDim.x, 0, n0[h], n1[h]);
        }
        ok = warp_wait(smem_addr(&sm->bempty[slot]), ((a / FTC_BSLOTS) & 1u) ^ 1u, err, ATC_ERR);
        if (!ok) break;
        unsigned char* bt = bring + slot * bslot;
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (live[h])
            split3_store8(x[h], bt + off[h], bt + NR * 32 + off[h], bt + 2 * NR * 32 + off[h]);
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&sm->bfull[slot]));
      }
    }
  } else {
    // ---------------- epilogue ----------------
    const int q4 = warp & 3;                                    // TMEM lane quarter
    const int L = 32 * q4 + lane, m = L >> 1, c = L & 1;
    const bool live = m < M;
    const int et = threadIdx.x - 32 * (2 + FTC_CONV_WARPS);     // 0..FTC_EPI-1
    const int KH = (K + 1) / 2, klo = (et >= 128) ? KH : 0;     // this warp's levels
    const int khi = (et >= 128) ? K : KH;
    const int SS = ftc_stage_stride(K);
    unsigned ul = 0;
    for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x, ++ul) {
      const int e = u / J, j = u - e * J;
      // the table carries the 1 / I of the forward transform
      const float wg = d.jfac[JF_GW * J + j];
      const float wd = d.jfac[JF_GWDELC * J + j];
      const float wdm = wd * float(m);
      const int b = ul & 1;
      ok = warp_wait(smem_addr(&sm->accfull[b]), (ul >> 1) & 1u, err, ATC_ERR);
      // one decision for the eight epilogue warps (a named-barrier OR), which
      // also orders this unit's staging writes after every thread's copy-out
      // of the previous unit
      unsigned bad;
      asm volatile(
          "{\n\t.reg .pred pb, po;\n\t"
          "setp.eq.u32 pb, %1, 0;\n\t"
          "bar.red.or.pred po, 1, 256, pb;\n\t"
          "selp.u32 %0, 1, 0, po;\n\t}\n"
          : "=r"(bad)
          : "r"(ok ? 1u : 0u)
          : "memory");
      if (bad) {
        ok = false;
        break;
      }
      tc_fence_after();
      const unsigned tl = tbase + ((unsigned)(32 * q4) << 16) + (unsigned)(b * NR);
      for (int k = klo; k < khi; ++k) {
        unsigned r[9];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%9];\n"
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%1}, [%10];\n"
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%2}, [%11];\n"
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%3}, [%12];\n"
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%4}, [%13];\n"
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%5}, [%14];\n"
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%6}, [%15];\n"
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%7}, [%16];\n"
            "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%8}, [%17];\n"
            "tcgen05.wait::ld.sync.aligned;\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
              "=r"(r[6]), "=r"(r[7]), "=r"(r[8])
            : "r"(tl + (unsigned)(0 * K + k)), "r"(tl + (unsigned)(1 * K + k)),
              "r"(tl + (unsigned)(2 * K + k)), "r"(tl + (unsigned)(3 * K + k)),
              "r"(tl + (unsigned)(4 * K + k)), "r"(tl + (unsigned)(5 * K + k)),
              "r"(tl + (unsigned)(6 * K + k)), "r"(tl + (unsigned)(7 * K + k)),
              "r"(tl + (unsigned)(8 * K + k))
            : "memory");
        float v[9];
#pragma unroll
        for (int f = 0; f < 9; ++f) v[f] = __uint_as_float(r[f]);
        // rows gt xu g yu fu fv ke xv yv; the partner lane holds the other
        // part (Re <-> Im) of xu and yu for the i m terms
        const float pxu = __shfl_xor_sync(0xffffffffu, v[1], 1);
        const float pyu = __shfl_xor_sync(0xffffffffu, v[3], 1);
        const float sg = c ? -1.f : 1.f;        // Re: + wdm Im(xu); Im: - wdm Re(xu)
        if (live) {
          float* o = stage + (size_t)m * SS + (k * AF_N) * 2 + c;
          o[2 * AF_T] = wg * v[0] + sg * wdm * pxu;
          o[2 * AF_Q] = wg * v[2] + sg * wdm * pyu;
          o[2 * AF_FU] = wd * v[4];
          o[2 * AF_FV] = wd * v[5];
          o[2 * AF_KE] = wg * v[6];
          o[2 * AF_XV] = wd * v[7];
          o[2 * AF_YV] = wd * v[8];
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_addr(&sm->accempty[b]));
      asm volatile("bar.sync 1, 256;\n" ::: "memory");
      // staged rows -> af: for each m, K * 7 complex contiguous
      const int rowf = K * AF_N * 2;                       // floats per m
      const int nq = rowf / 4;                             // float4 per m
      const int n4 = M * nq;
      float* afe = reinterpret_cast<float*>(d.af) + (((size_t)e * M) * J + j) * rowf;
      for (int x = et; x < n4; x += FTC_EPI) {
        const int mm = x / nq, w = x - mm * nq;
        *reinterpret_cast<float4*>(afe + (size_t)mm * J * rowf + 4 * w) =
            *reinterpret_cast<const float4*>(stage + (size_t)mm * SS + 4 * w);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tbase, (unsigned)pl.tcols);
  }
}

// Surface rows (gt_pi, pi(t - dt)) of the longitude analysis on the FMA
// pipes, rounded to nearest: one block per (latitude, FSURF_EB members), one
// thread per lane L = 2m + c; W[L][i] read from an FP32 cos table (the sine
// as cos(theta + pi / 2)), the members' rows staged [row][i][member] so that
// a table value feeds 2 x FSURF_EB FMAs.  Writes afs = gw / I X, as k_fdft.
constexpr int FSURF_EB = 8;

inline size_t fsurf_smem(int I) { return sizeof(float) * (size_t)I * (1 + 2 * FSURF_EB); }

__global__ void __launch_bounds__(128) k_fdft_surf(SD<float> d, const float* __restrict__ cs) {
  extern __shared__ float4 sh_fsurf[];
  float* tw = reinterpret_cast<float*>(sh_fsurf);
  const int I = d.I, J = d.J, M = d.M, E = d.E, R = 2 + 9 * d.K;
  float* rows = tw + I;                                  // [2][I][FSURF_EB]
  const int j = blockIdx.x, e0 = blockIdx.y * FSURF_EB;
  for (int t = threadIdx.x; t < I; t += blockDim.x) tw[t] = cs[t];
  for (int x = threadIdx.x; x < 2 * I * FSURF_EB; x += blockDim.x) {
    const int eb = x / (2 * I), rem = x - eb * 2 * I, r = rem / I, i = rem - r * I;
    const int e = e0 + eb;
    rows[(r * I + i) * FSURF_EB + eb] =
        e < E ? d.grid9[(((size_t)e * J + j) * R + r) * I + i] : 0.f;
  }
  __syncthreads();
  const int L = threadIdx.x, m = L >> 1, c = L & 1;
  if (m >= M) return;
  const int off = c ? I / 4 : 0;                         // -sin(t) = cos(t + pi / 2)
  float acc[2][FSURF_EB];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int b = 0; b < FSURF_EB; ++b) acc[h][b] = 0.f;
  for (int i = 0; i < I; ++i) {
    const float w = tw[(m * i + off) & (I - 1)];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float4* p = reinterpret_cast<const float4*>(rows + (size_t)(h * I + i) * FSURF_EB);
#pragma unroll
      for (int q = 0; q < FSURF_EB / 4; ++q) {
        const float4 v = p[q];
        acc[h][4 * q] = fmaf(w, v.x, acc[h][4 * q]);
        acc[h][4 * q + 1] = fmaf(w, v.y, acc[h][4 * q + 1]);
        acc[h][4 * q + 2] = fmaf(w, v.z, acc[h][4 * q + 2]);
        acc[h][4 * q + 3] = fmaf(w, v.w, acc[h][4 * q + 3]);
      }
    }
  }
  const float wg = d.jfac[JF_GW * J + j] / float(I);
#pragma unroll
  for (int b = 0; b < FSURF_EB; ++b) {
    const int e = e0 + b;
    if (e < E) {
      float* os = reinterpret_cast<float*>(d.afs) + ((((size_t)e * M + m) * J + j) * 2) * 2 + c;
      os[0] = wg * acc[0][b];
      os[2] = wg * acc[1][b];
    }
  }
}

}  // namespace lbm
