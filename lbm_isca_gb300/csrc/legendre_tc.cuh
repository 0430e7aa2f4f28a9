// Legendre analysis of the FP32 stepper on the tensor cores (tcgen05), with
// bfloat16 split-precision operands and FP32 accumulation in tensor memory.
//
// Per wavenumber m and member group, the explicit tendencies of rows
// n = m..N are the latitude sums of Legendre.analysis in k_anal, as products
//   D[lane][n] = sum_j A[lane][j] T[n][j]
// with lanes = (member of the group, level k, Re|Im) -- up to 128 rows of
// one MMA -- and j over all latitudes (the tensor cores need no equatorial
// fold).  Nine A matrices (fields of af, two of them multiplied by i m,
// which swaps Re and Im of a level) meet one table each (P, H or nn1a P)
// and accumulate into four TMEM regions, one per tendency:
//   vor = (i m FV) P + FU H
//   div = (i m FU) P + (-FV) H + KE (nn1a P)
//   T   = T P + XV H,        q = Q P + YV H
// (the sums of k_anal, spectral.py:190, 227-244 / dynamics.py:237-262).
//
// Operands are FP32 values split three ways into bfloat16 (tc_common.cuh);
// the MMA chain sums 6 products per pair (b0 c0 .. down to third order,
// FP32-level products) or 3 (b0 c0 + b0 c1 + b1 c0, about 16 bits).  The
// tables are split once from FP64 on the host side, and laid out as TMA
// images: per (m, 16-latitude step) the 3 tables x 3 pieces in the K-major
// tile layout, one bulk copy each.
//
// Roles of the persistent CTA (one per SM):
//   warp 0        bulk copies: a step's af rows of the group's members (one
//                 contiguous run per member) and its table image, into a
//                 two-stage ring;
//   warp 1        TMEM allocation and the MMA issue (one thread);
//   warps 2..17   conversion: staged FP32 af -> the nine split A tiles, six
//                 A slots in a ring; warps 2..9 take the even tiles, 10..17
//                 the odd ones;
//   warps 18..21  epilogue: tcgen05.ld of the four regions -> tend.
// Every wait is bounded (tc::mbar_wait); a timeout sets bit 2 of *err and
// the CTA winds down without leaving copies or MMAs in flight.
#pragma once
#include "tc_common.cuh"

namespace lbm {

constexpr int ATC_STAGES = 2;
constexpr int ATC_ASLOTS = 6;
constexpr int ATC_CONV_WARPS = 16;     // two groups of 8: even / odd A matrices
constexpr int ATC_THREADS = 32 * (2 + ATC_CONV_WARPS + 4);
constexpr int ATC_NMAT = 9;
constexpr int ATC_ERR = 2;            // *err bit set by a timed-out wait

LBM_HD int atc_nb(int N, int m) { return ((N + 1 - m) + 15) / 16 * 16; }

// Launch plan of the tensor-core analysis (host and device).
struct AtcPlan {
  int G, ngroups, nunits, KS, NB, nacc, tcols;
  unsigned data_bytes, tab_bytes, stage_bytes, a_bytes, smem;
};

// gcap > 0 caps the members per MMA tile (a tuning choice: fewer members,
// more units of work).
LBM_HD AtcPlan atc_plan(int E, int J, int K, int N, int gcap = 0) {
  AtcPlan p;
  p.G = 128 / (2 * K);
  if (gcap > 0 && p.G > gcap) p.G = gcap;
  if (p.G < 1) p.G = 1;
  if (p.G > E) p.G = E;
  p.ngroups = (E + p.G - 1) / p.G;
  p.nunits = (N + 1) * p.ngroups;
  p.KS = J / 16;
  p.NB = atc_nb(N, 0);
  p.nacc = (8 * p.NB <= 512) ? 2 : 1;
  const int cols = p.nacc * 4 * p.NB;
  p.tcols = cols <= 32 ? 32 : cols <= 64 ? 64 : cols <= 128 ? 128 : cols <= 256 ? 256 : 512;
  p.data_bytes = (unsigned)(p.G * 16 * K * 7 * 8);
  p.tab_bytes = (unsigned)(9 * p.NB * 32);
  p.stage_bytes = ((p.data_bytes + 1023) / 1024 + (p.tab_bytes + 1023) / 1024) * 1024;
  p.a_bytes = 3 * 4096;
  // barriers (2 S + 2 R + 2 acc + done) and the TMEM slot, then 1 KB alignment
  p.smem = 1024 + ATC_STAGES * p.stage_bytes + ATC_ASLOTS * p.a_bytes + 1024;
  return p;
}

// Byte offset of wavenumber m's table image: sum over m' < m of KS * 9 * NB(m') * 32.
LBM_HD size_t atc_tab_offset(int N, int KS, int m) {
  size_t o = 0;
  for (int q = 0; q < m; ++q) o += (size_t)KS * 9 * atc_nb(N, q) * 32;
  return o;
}

struct AtcSmem {
  unsigned long long full[ATC_STAGES], empty[ATC_STAGES], afull[ATC_ASLOTS],
      aempty[ATC_ASLOTS], accfull[2], accempty[2], done;
  unsigned tslot;
};

// A matrix am = 0..8: (i m FV) P, FU H -> vor; (i m FU) P, (-FV) H, KE (nn1a P)
// -> div; T P, XV H -> T; Q P, YV H -> q.  Tables 0 = P, 1 = H, 2 = nn1a P;
// regions 0 = vor, 1 = div, 2 = T, 3 = q.  The split pieces (A, table) of
// the six products, smallest first, are (2,0) (1,1) (0,2) (1,0) (0,1)
// (0,0); the last three are the two-way (three-product) form.

// A matrix AM -> (table, region) at compile time (the same as the tables above).
template <int AM> struct AtcMat {
  static constexpr int tab = AM == 1 || AM == 3 || AM == 6 || AM == 8 ? 1 : AM == 4 ? 2 : 0;
  static constexpr int reg = AM < 2 ? 0 : AM < 5 ? 1 : AM < 7 ? 2 : 3;
  static constexpr int field = AM == 0 || AM == 3 ? AF_FV : AM == 1 || AM == 2 ? AF_FU
                             : AM == 4 ? AF_KE : AM == 5 ? AF_T : AM == 6 ? AF_XV
                             : AM == 7 ? AF_Q : AF_YV;
  static constexpr bool swap = AM == 0 || AM == 2;     // times i m: Re and Im swap
  static constexpr bool neg = AM == 3;
};

// One thread's part of A tile AM: the 8 latitudes of chunk ch of row
// (member, level, ri), read from the staged af rows (stride jst floats) and
// split into the tile's three pieces.
template <int AM>
LBM_D void atc_convert(const float* rows, size_t jst, int ri, float rm, unsigned char* at,
                       unsigned off) {
  using T = AtcMat<AM>;
  const int c = 2 * T::field + (T::swap ? 1 - ri : ri);
  const float sc = T::swap ? (ri ? rm : -rm) : (T::neg ? -1.0f : 1.0f);
  float x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = (T::swap || T::neg) ? sc * rows[q * jst + c]
                                                          : rows[q * jst + c];
  tc::split3_store8(x, at + off, at + 4096 + off, at + 8192 + off);
}
LBM_D void atc_convert_any(int am, const float* rows, size_t jst, int ri, float rm,
                           unsigned char* at, unsigned off) {
  switch (am) {
    case 0: atc_convert<0>(rows, jst, ri, rm, at, off); break;
    case 1: atc_convert<1>(rows, jst, ri, rm, at, off); break;
    case 2: atc_convert<2>(rows, jst, ri, rm, at, off); break;
    case 3: atc_convert<3>(rows, jst, ri, rm, at, off); break;
    case 4: atc_convert<4>(rows, jst, ri, rm, at, off); break;
    case 5: atc_convert<5>(rows, jst, ri, rm, at, off); break;
    case 6: atc_convert<6>(rows, jst, ri, rm, at, off); break;
    case 7: atc_convert<7>(rows, jst, ri, rm, at, off); break;
    default: atc_convert<8>(rows, jst, ri, rm, at, off); break;
  }
}

// The MMAs of one A tile AM: the split products (smallest first, from q0)
// into its region; `initm` marks the regions already written in this unit.
template <int AM>
LBM_D void atc_issue(unsigned dbase, int NB, uint64_t adesc, uint64_t bdesc0, unsigned tstride,
                     unsigned idesc, int q0, unsigned& initm) {
  using T = AtcMat<AM>;
  const unsigned dcol = dbase + (unsigned)(T::reg * NB);
  // descriptor address fields advance by (bytes >> 4)
  const uint64_t bt = bdesc0 + (uint64_t)((T::tab * 3 * tstride) >> 4);
  bool acc = (initm >> T::reg) & 1u;
  const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    if (q < q0) continue;
    tc::mma_bf16(dcol, adesc + (uint64_t)((pa[q] * 4096u) >> 4),
             bt + (uint64_t)((pb[q] * tstride) >> 4), idesc, acc);
    acc = true;
  }
  initm |= 1u << T::reg;
}
LBM_D void atc_issue_any(int am, unsigned dbase, int NB, uint64_t adesc, uint64_t bdesc0,
                         unsigned tstride, unsigned idesc, int q0, unsigned& initm) {
  switch (am) {
    case 0: atc_issue<0>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 1: atc_issue<1>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 2: atc_issue<2>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 3: atc_issue<3>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 4: atc_issue<4>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 5: atc_issue<5>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 6: atc_issue<6>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 7: atc_issue<7>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
    default: atc_issue<8>(dbase, NB, adesc, bdesc0, tstride, idesc, q0, initm); break;
  }
}

__global__ void __launch_bounds__(ATC_THREADS, 1)
    k_anal_tc(SD<float> d, const unsigned char* __restrict__ tabs, AtcPlan pl, int nprod) {
  extern __shared__ unsigned char smraw_tc[];
  // 1 KB alignment by pointer arithmetic on the shared array itself, so
  // that every access below stays a shared-memory access (not generic)
  unsigned char* base = smraw_tc + ((1024u - (tc::smem_addr(smraw_tc) & 1023u)) & 1023u);
  AtcSmem* sm = reinterpret_cast<AtcSmem*>(base);
  unsigned char* stages = base + 1024;
  unsigned char* aring = stages + ATC_STAGES * pl.stage_bytes;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int E = d.E, J = d.J, K = d.K, N = d.N, M = d.M, KS = pl.KS, NB = pl.NB;
  int* err = d.err;
  using namespace tc;

  if (threadIdx.x == 0) {
    for (int i = 0; i < ATC_STAGES; ++i) {
      mbar_init(smem_addr(&sm->full[i]), 1);
      mbar_init(smem_addr(&sm->empty[i]), 1);
    }
    for (int i = 0; i < ATC_ASLOTS; ++i) {
      mbar_init(smem_addr(&sm->afull[i]), ATC_CONV_WARPS / 2);
      mbar_init(smem_addr(&sm->aempty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_addr(&sm->accfull[i]), 1);
      mbar_init(smem_addr(&sm->accempty[i]), 4);
    }
    mbar_init(smem_addr(&sm->done), 1);
    fence_mbar_init();
  }
  // unused lanes of the A tiles (rows past G 2K) stay zero
  for (int i = threadIdx.x; i < ATC_ASLOTS * (int)pl.a_bytes / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(aring)[i] = make_uint4(0, 0, 0, 0);
  fence_async_smem();
  if (warp == 1) tmem_alloc(smem_addr(&sm->tslot), (unsigned)pl.tcols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tbase = sm->tslot;
  bool ok = true;

  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      unsigned t = 0;
      const unsigned rowb = (unsigned)(16 * K * 7 * 8);
      for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x) {
        const int m = u / pl.ngroups, g = u - m * pl.ngroups;
        const int e0 = g * pl.G, gm = min(pl.G, E - e0);
        const int nb = atc_nb(N, m);
        const unsigned tb = 9u * nb * 32u;
        const unsigned char* tm = tabs + atc_tab_offset(N, KS, m);
        for (int s = 0; s < KS && ok; ++s, ++t) {
          const int st = t % ATC_STAGES;
          const unsigned ph = (t / ATC_STAGES) & 1u;
          ok = mbar_wait(smem_addr(&sm->empty[st]), ph ^ 1u, err, ATC_ERR);
          if (!ok) break;
          unsigned char* sd = stages + st * pl.stage_bytes;
          unsigned char* stab = sd + (pl.data_bytes + 1023) / 1024 * 1024;
          const unsigned bar = smem_addr(&sm->full[st]);
          mbar_expect_tx(bar, gm * rowb + tb);
          for (int mi = 0; mi < gm; ++mi) {
            const float* src = reinterpret_cast<const float*>(d.af) +
                               ((((size_t)(e0 + mi) * M + m) * J + s * 16) * K) * 14;
            bulk_g2s(smem_addr(sd + mi * rowb), src, rowb, bar);
          }
          bulk_g2s(smem_addr(stab), tm + (size_t)s * tb, tb, bar);
        }
      }
      // every copy issued has landed before the CTA winds down: wait for the
      // last fill of each stage (fills of stage st: st, st + S, ... < t)
      for (int st = 0; st < ATC_STAGES; ++st) {
        const unsigned fills = t / ATC_STAGES + ((unsigned)st < t % ATC_STAGES ? 1u : 0u);
        if (fills) mbar_wait(smem_addr(&sm->full[st]), (fills - 1) & 1u, err, ATC_ERR);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      const int q0 = nprod == 3 ? 3 : 0;
      unsigned t = 0, a = 0, ul = 0;
      for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x, ++ul) {
        const int m = u / pl.ngroups;
        const int nb = atc_nb(N, m);
        const unsigned idesc = idesc_bf16(128, nb);
        const int b = ul % pl.nacc;
        ok = mbar_wait(smem_addr(&sm->accempty[b]), ((ul / pl.nacc) & 1u) ^ 1u, err, ATC_ERR);
        if (!ok) break;
        tc_fence_after();
        const unsigned dbase = tbase + (unsigned)(b * 4 * NB);
        unsigned initm = 0;
        const unsigned tstride = (unsigned)nb * 32u;
        for (int s = 0; s < KS && ok; ++s, ++t) {
          const int st = t % ATC_STAGES;
          ok = mbar_wait(smem_addr(&sm->full[st]), (t / ATC_STAGES) & 1u, err, ATC_ERR);
          if (!ok) break;
          const unsigned char* sd = stages + st * pl.stage_bytes;
          const uint64_t bdesc0 = smem_desc(smem_addr(sd + (pl.data_bytes + 1023) / 1024 * 1024));
          for (int am = 0; am < ATC_NMAT; ++am, ++a) {
            const int slot = a % ATC_ASLOTS;
            ok = mbar_wait(smem_addr(&sm->afull[slot]), (a / ATC_ASLOTS) & 1u, err, ATC_ERR);
            if (!ok) break;
            tc_fence_after();
            atc_issue_any(am, dbase, NB, smem_desc(smem_addr(aring + slot * pl.a_bytes)), bdesc0,
                          tstride, idesc, q0, initm);
            mma_commit(smem_addr(&sm->aempty[slot]));
          }
          if (!ok) break;
          mma_commit(smem_addr(&sm->empty[st]));
        }
        if (!ok) break;
        mma_commit(smem_addr(&sm->accfull[b]));
      }
      // every MMA issued has completed before the teardown
      mma_commit(smem_addr(&sm->done));
      mbar_wait(smem_addr(&sm->done), 0, err, ATC_ERR);
    }
  } else if (warp < 2 + ATC_CONV_WARPS) {
    // ---------------- conversion ----------------
    const int ct = threadIdx.x - 64;
    const int grp = ct >> 8;                      // 0: even A matrices, 1: odd
    const int row = ct & 127, ch = (ct >> 7) & 1;   // A row, 8-latitude chunk
    const int twoK = 2 * K;
    const int mi = row / twoK, rem = row - mi * twoK, k = rem >> 1, ri = rem & 1;
    unsigned t = 0, a = 0;
    for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x) {
      const int m = u / pl.ngroups, g = u - m * pl.ngroups;
      const int gm = min(pl.G, E - g * pl.G);
      const bool live = mi < gm;
      const float rm = (float)m;
      for (int s = 0; s < KS && ok; ++s, ++t) {
        const int st = t % ATC_STAGES;
        ok = warp_wait(smem_addr(&sm->full[st]), (t / ATC_STAGES) & 1u, err, ATC_ERR);
        if (!ok) break;
        const float* sd = reinterpret_cast<const float*>(stages + st * pl.stage_bytes);
        // the 8 staged rows of this thread's chunk: (member mi, latitude, level k)
        const float* rows = sd + ((size_t)(mi * 16 + ch * 8) * K + k) * 14;
        const size_t jst = (size_t)K * 14;
        for (int am = grp; am < ATC_NMAT; am += 2) {
          const unsigned aa = a + (unsigned)am;      // this tile's place in the A ring
          const int slot = aa % ATC_ASLOTS;
          ok = warp_wait(smem_addr(&sm->aempty[slot]), ((aa / ATC_ASLOTS) & 1u) ^ 1u, err,
                         ATC_ERR);
          if (!ok) break;
          if (live)
            atc_convert_any(am, rows, jst, ri, rm, aring + slot * pl.a_bytes,
                            tile_offset(row, ch * 8));
          fence_async_smem();
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_addr(&sm->afull[slot]));
        }
        a += ATC_NMAT;
      }
    }
  } else {
    // ---------------- epilogue ----------------
    const int q4 = warp & 3;
    const int row = 32 * q4 + lane;
    const int twoK = 2 * K;
    const int mi = row / twoK, rem = row - mi * twoK, k = rem >> 1, ri = rem & 1;
    const int NS = d.NS;
    float* tend = reinterpret_cast<float*>(d.tend);
    unsigned ul = 0;
    for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x, ++ul) {
      const int m = u / pl.ngroups, g = u - m * pl.ngroups;
      const int e = g * pl.G + mi;
      const bool live = (mi < pl.G) && (e < E);
      const int nr = N + 1 - m, nb = atc_nb(N, m);
      const int b = ul % pl.nacc;
      ok = warp_wait(smem_addr(&sm->accfull[b]), (ul / pl.nacc) & 1u, err, ATC_ERR);
      if (!ok) break;
      tc_fence_after();
      const unsigned tl = tbase + ((unsigned)(32 * q4) << 16) + (unsigned)(b * 4 * NB);
      const size_t off = (size_t)spec_offset(m, N);
      for (int reg = 0; reg < 4; ++reg) {
        float* dst = tend + ((((size_t)e * 4 + reg) * NS + off) * K + k) * 2 + ri;
        for (int c0 = 0; c0 < nb; c0 += 16) {
          float v[16];
          tmem_ld16(tl + (unsigned)(reg * NB + c0), v);
          if (live) {
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (c0 + i < nr) dst[(size_t)(c0 + i) * K * 2] = v[i];
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_addr(&sm->accempty[b]));
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

}  // namespace lbm
