// Legendre synthesis of the FP32 stepper on the tensor cores (tcgen05),
// bfloat16 split operands, FP32 accumulation in tensor memory: the level
// fields of sf (k_synth's wind and scalar terms) as products
//   D[lane][j] = sum_n A[lane][n] T[j][n]
// with lanes = (member of the group, level k, Re|Im), n = m..N in steps of
// 16, and j over a part of the latitudes (all of them when six regions of J
// columns fit the tensor memory, else two halves).  Six A tiles per step,
// from the state's vor, div, T, q; the factors i m and the inverse
// Laplacian live in the tables:
//   U   = (i div) (m P il) + vor (-H il)      [u cos, spectral.py:256-276]
//   V   = (i vor) (m P il) + div (H il)
//   VOR = vor P,  DIV = div P,  T = T P,  Q = q P
// where (i X) swaps Re and Im of a level (the thread holding X.im writes
// -X.im into the Re row of the swapped tile, the one holding X.re writes
// it into the Im row: a sign change of the split pieces, no second split).
//
// Roles (one persistent CTA per SM), as in the analysis (legendre_tc.cuh):
// warp 0 bulk copies (the step's rows n of the group's four state fields,
// and the table image of (m, step, part)); warp 1 TMEM and MMA issue; warps
// 2..17 conversion (warps 2..9: vor and T, 10..17: div and q); warps 18..21
// the epilogue, which writes sf rows through a partner exchange so that each
// warp stores whole 768-byte runs.  The surface fields of sfs stay with the
// FMA kernel (k_synth, surface part only).
#pragma once
#include "tc_common.cuh"

namespace lbm {

constexpr int STC_STAGES = 2;
constexpr int STC_ASLOTS = 6;
constexpr int STC_CONV_WARPS = 16;
constexpr int STC_THREADS = 32 * (2 + STC_CONV_WARPS + 4);
constexpr int STC_NTILE = 6;          // vor, i vor, div, i div, T, q
constexpr int STC_NTAB = 4;           // m P il, -H il, H il, P
constexpr int STC_NREG = 6;           // U, V, VOR, DIV, T, Q

LBM_HD int stc_ks(int N, int m) { return (N + 1 - m + 15) / 16; }

struct StcPlan {
  int G, ngroups, nparts, JT, nunits, nacc, tcols;
  unsigned data_bytes, tab_bytes, stage_bytes, a_bytes, smem;
};

LBM_HD StcPlan stc_plan(int E, int J, int K, int N, int gcap = 0) {
  StcPlan p;
  p.G = 128 / (2 * K);
  if (gcap > 0 && p.G > gcap) p.G = gcap;
  if (p.G < 1) p.G = 1;
  if (p.G > E) p.G = E;
  p.ngroups = (E + p.G - 1) / p.G;
  p.nparts = (STC_NREG * J <= 512) ? 1 : 2;
  p.JT = J / p.nparts;
  p.nunits = (N + 1) * p.nparts * p.ngroups;
  p.nacc = (2 * STC_NREG * p.JT <= 512) ? 2 : 1;
  const int cols = p.nacc * STC_NREG * p.JT;
  p.tcols = cols <= 32 ? 32 : cols <= 64 ? 64 : cols <= 128 ? 128 : cols <= 256 ? 256 : 512;
  p.data_bytes = (unsigned)(p.G * 4 * 16 * K * 8);
  p.tab_bytes = (unsigned)(STC_NTAB * 3 * p.JT * 32);
  p.stage_bytes = ((p.data_bytes + 1023) / 1024 + (p.tab_bytes + 1023) / 1024) * 1024;
  p.a_bytes = 3 * 4096;
  p.smem = 1024 + STC_STAGES * p.stage_bytes + STC_ASLOTS * p.a_bytes + 1024;
  return p;
}

// Byte offset of the table image of (m, part): per m, per part, per step s,
// STC_NTAB tables x 3 pieces of JT x 16 tiles.
LBM_HD size_t stc_tab_offset(int N, int nparts, int JT, int m, int part) {
  size_t o = 0;
  for (int q = 0; q < m; ++q) o += (size_t)nparts * stc_ks(N, q);
  o += (size_t)part * stc_ks(N, m);
  return o * STC_NTAB * 3 * JT * 32;
}

struct StcSmem {
  unsigned long long full[STC_STAGES], empty[STC_STAGES], afull[STC_ASLOTS],
      aempty[STC_ASLOTS], accfull[2], accempty[2], done;
  unsigned tslot;
};

// The MMAs of tile TL (regions, tables): 0 vor -> U (-H il), VOR (P);
// 1 i vor -> V (m P il); 2 div -> V (H il), DIV (P); 3 i div -> U (m P il);
// 4 T -> T (P); 5 q -> Q (P).
template <int TL>
LBM_D void stc_issue(unsigned dbase, int JT, uint64_t adesc, uint64_t bdesc0, unsigned tstride,
                     unsigned idesc, int q0, unsigned& initm) {
  constexpr int npair = (TL == 0 || TL == 2) ? 2 : 1;
  constexpr int reg[2] = {TL == 0 ? 0 : TL == 1 ? 1 : TL == 2 ? 1 : TL == 3 ? 0 : TL == 4 ? 4 : 5,
                          TL == 0 ? 2 : 3};
  constexpr int tab[2] = {TL == 0 ? 1 : TL == 1 ? 0 : TL == 2 ? 2 : TL == 3 ? 0 : 3, 3};
  const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
  for (int pr = 0; pr < npair; ++pr) {
    const unsigned dcol = dbase + (unsigned)(reg[pr] * JT);
    const uint64_t bt = bdesc0 + (uint64_t)((tab[pr] * 3 * tstride) >> 4);
    bool acc = (initm >> reg[pr]) & 1u;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      if (q < q0) continue;
      tc::mma_bf16(dcol, adesc + (uint64_t)((pa[q] * 4096u) >> 4),
                   bt + (uint64_t)((pb[q] * tstride) >> 4), idesc, acc);
      acc = true;
    }
    initm |= 1u << reg[pr];
  }
}
LBM_D void stc_issue_any(int tl, unsigned dbase, int JT, uint64_t adesc, uint64_t bdesc0,
                         unsigned tstride, unsigned idesc, int q0, unsigned& initm) {
  switch (tl) {
    case 0: stc_issue<0>(dbase, JT, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 1: stc_issue<1>(dbase, JT, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 2: stc_issue<2>(dbase, JT, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 3: stc_issue<3>(dbase, JT, adesc, bdesc0, tstride, idesc, q0, initm); break;
    case 4: stc_issue<4>(dbase, JT, adesc, bdesc0, tstride, idesc, q0, initm); break;
    default: stc_issue<5>(dbase, JT, adesc, bdesc0, tstride, idesc, q0, initm); break;
  }
}

// 8 consecutive FP32 columns of this thread's TMEM lane.
LBM_D void tmem_ld8(unsigned taddr, float* v) {
  unsigned r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(STC_THREADS, 1)
    k_synth_tc(SD<float> d, const unsigned char* __restrict__ tabs, StcPlan pl, int nprod) {
  extern __shared__ unsigned char smraw_stc[];
  // 1 KB alignment by pointer arithmetic on the shared array itself, so
  // that every access below stays a shared-memory access (not generic)
  unsigned char* base = smraw_stc + ((1024u - (tc::smem_addr(smraw_stc) & 1023u)) & 1023u);
  StcSmem* sm = reinterpret_cast<StcSmem*>(base);
  unsigned char* stages = base + 1024;
  unsigned char* aring = stages + STC_STAGES * pl.stage_bytes;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int E = d.E, J = d.J, K = d.K, N = d.N, M = d.M, NS = d.NS, JT = pl.JT;
  const unsigned tab_off = (pl.data_bytes + 1023) / 1024 * 1024;   // tables within a stage
  int* err = d.err;
  using namespace tc;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STC_STAGES; ++i) {
      mbar_init(smem_addr(&sm->full[i]), 1);
      mbar_init(smem_addr(&sm->empty[i]), 1);
    }
    for (int i = 0; i < STC_ASLOTS; ++i) {
      mbar_init(smem_addr(&sm->afull[i]), STC_CONV_WARPS / 2);
      mbar_init(smem_addr(&sm->aempty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_addr(&sm->accfull[i]), 1);
      mbar_init(smem_addr(&sm->accempty[i]), 4);
    }
    mbar_init(smem_addr(&sm->done), 1);
    fence_mbar_init();
  }
  for (int i = threadIdx.x; i < STC_ASLOTS * (int)pl.a_bytes / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(aring)[i] = make_uint4(0, 0, 0, 0);
  fence_async_smem();
  if (warp == 1) tmem_alloc(smem_addr(&sm->tslot), (unsigned)pl.tcols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tbase = sm->tslot;
  bool ok = true;
  // unit u -> (m, part, group)
  auto unit = [&](int u, int& m, int& part, int& g) {
    g = u % pl.ngroups;
    const int mp = u / pl.ngroups;
    part = mp % pl.nparts;
    m = mp / pl.nparts;
  };

  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      unsigned t = 0;
      const unsigned rowb = (unsigned)(K * 8);        // one (n) row of K complex
      const unsigned tb = pl.tab_bytes;
      for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x) {
        int m, part, g;
        unit(u, m, part, g);
        const int e0 = g * pl.G, gm = min(pl.G, E - e0);
        const int ks = stc_ks(N, m), nr = N + 1 - m;
        const unsigned char* tm = tabs + stc_tab_offset(N, pl.nparts, JT, m, part);
        const size_t off = (size_t)spec_offset(m, N);
        for (int s = 0; s < ks && ok; ++s, ++t) {
          const int st = t % STC_STAGES;
          ok = mbar_wait(smem_addr(&sm->empty[st]), ((t / STC_STAGES) & 1u) ^ 1u, err, ATC_ERR);
          if (!ok) break;
          unsigned char* sd = stages + st * pl.stage_bytes;
          const unsigned bar = smem_addr(&sm->full[st]);
          const int nv = min(16, nr - 16 * s);
          mbar_expect_tx(bar, gm * 4 * nv * rowb + tb);
          for (int mi = 0; mi < gm; ++mi)
            for (int f = 0; f < 4; ++f) {
              const float* src = reinterpret_cast<const float*>(d.sa3) +
                                 ((((size_t)(e0 + mi) * 4 + f) * NS + off + 16 * s) * K) * 2;
              bulk_g2s(smem_addr(sd + (mi * 4 + f) * 16 * rowb), src, nv * rowb, bar);
            }
          bulk_g2s(smem_addr(sd + tab_off), tm + (size_t)s * tb, tb, bar);
        }
      }
      for (int st = 0; st < STC_STAGES; ++st) {
        const unsigned fills = t / STC_STAGES + ((unsigned)st < t % STC_STAGES ? 1u : 0u);
        if (fills) mbar_wait(smem_addr(&sm->full[st]), (fills - 1) & 1u, err, ATC_ERR);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      const int q0 = nprod == 3 ? 3 : 0;
      const unsigned idesc = idesc_bf16(128, JT);
      const unsigned tstride = (unsigned)JT * 32u;
      unsigned t = 0, a = 0, ul = 0;
      for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x, ++ul) {
        int m, part, g;
        unit(u, m, part, g);
        const int ks = stc_ks(N, m);
        const int b = ul % pl.nacc;
        ok = mbar_wait(smem_addr(&sm->accempty[b]), ((ul / pl.nacc) & 1u) ^ 1u, err, ATC_ERR);
        if (!ok) break;
        tc_fence_after();
        const unsigned dbase = tbase + (unsigned)(b * STC_NREG * JT);
        unsigned initm = 0;
        for (int s = 0; s < ks && ok; ++s, ++t) {
          const int st = t % STC_STAGES;
          ok = mbar_wait(smem_addr(&sm->full[st]), (t / STC_STAGES) & 1u, err, ATC_ERR);
          if (!ok) break;
          const uint64_t bdesc0 = smem_desc(smem_addr(stages + st * pl.stage_bytes + tab_off));
          for (int tl = 0; tl < STC_NTILE; ++tl, ++a) {
            const int slot = a % STC_ASLOTS;
            ok = mbar_wait(smem_addr(&sm->afull[slot]), (a / STC_ASLOTS) & 1u, err, ATC_ERR);
            if (!ok) break;
            tc_fence_after();
            stc_issue_any(tl, dbase, JT, smem_desc(smem_addr(aring + slot * pl.a_bytes)), bdesc0,
                          tstride, idesc, q0, initm);
            mma_commit(smem_addr(&sm->aempty[slot]));
          }
          if (!ok) break;
          mma_commit(smem_addr(&sm->empty[st]));
        }
        if (!ok) break;
        mma_commit(smem_addr(&sm->accfull[b]));
      }
      mma_commit(smem_addr(&sm->done));
      mbar_wait(smem_addr(&sm->done), 0, err, ATC_ERR);
    }
  } else if (warp < 2 + STC_CONV_WARPS) {
    // ---------------- conversion ----------------
    // group 0: vor (tiles 0, 1) then T (tile 4); group 1: div (2, 3) then q (5)
    const int ct = threadIdx.x - 64;
    const int grp = ct >> 8;
    const int row = ct & 127, ch = (ct >> 7) & 1;       // A row, 8-n chunk
    const int twoK = 2 * K;
    const int mi = row / twoK, rem = row - mi * twoK, k = rem >> 1, ri = rem & 1;
    const unsigned off = tile_offset(row, ch * 8), offs = tile_offset(row ^ 1, ch * 8);
    const unsigned neg = ri ? 0x80008000u : 0u;       // (i X): the Im row's value, negated
    unsigned t = 0, a = 0;
    for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x) {
      int m, part, g;
      unit(u, m, part, g);
      const int gm = min(pl.G, E - g * pl.G);
      const bool live = mi < gm;
      const int ks = stc_ks(N, m), nr = N + 1 - m;
      for (int s = 0; s < ks && ok; ++s, ++t) {
        const int st = t % STC_STAGES;
        ok = warp_wait(smem_addr(&sm->full[st]), (t / STC_STAGES) & 1u, err, ATC_ERR);
        if (!ok) break;
        const float* sd = reinterpret_cast<const float*>(stages + st * pl.stage_bytes);
        const int n0 = 16 * s + ch * 8;                  // first row n - m of the chunk
        for (int pass = 0; pass < 2 && ok; ++pass) {
          // pass 0: vor / div (a tile and its (i X) tile), pass 1: T / q
          const int f = pass == 0 ? grp : 2 + grp;
          const int tl = pass == 0 ? 2 * grp : 4 + grp;
          const int nt = pass == 0 ? 2 : 1;
          const unsigned aa = a + (unsigned)tl;
          for (int x = 0; x < nt && ok; ++x) {
            const unsigned ax = aa + (unsigned)x;
            ok = warp_wait(smem_addr(&sm->aempty[ax % STC_ASLOTS]),
                           ((ax / STC_ASLOTS) & 1u) ^ 1u, err, ATC_ERR);
          }
          if (!ok) break;
          unsigned char* at = aring + (aa % STC_ASLOTS) * pl.a_bytes;
          unsigned char* as = aring + ((aa + 1) % STC_ASLOTS) * pl.a_bytes;
          if (live) {
            const float* src = sd + ((size_t)(mi * 4 + f) * 16 * K + k) * 2 + ri;
            unsigned w[3][4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int na = n0 + 2 * q, nb = na + 1;
              const float xa = na < nr ? src[(size_t)(na - 16 * s) * K * 2] : 0.f;
              const float xb = nb < nr ? src[(size_t)(nb - 16 * s) * K * 2] : 0.f;
              unsigned p3[3];
              split3_pair(xa, xb, p3);
#pragma unroll
              for (int p = 0; p < 3; ++p) w[p][q] = p3[p];
            }
#pragma unroll
            for (int p = 0; p < 3; ++p)
              *reinterpret_cast<uint4*>(at + p * 4096 + off) =
                  make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
            if (nt == 2) {
#pragma unroll
              for (int p = 0; p < 3; ++p)
                *reinterpret_cast<uint4*>(as + p * 4096 + offs) =
                    make_uint4(w[p][0] ^ neg, w[p][1] ^ neg, w[p][2] ^ neg, w[p][3] ^ neg);
            }
          }
          fence_async_smem();
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(smem_addr(&sm->afull[aa % STC_ASLOTS]));
            if (nt == 2) mbar_arrive(smem_addr(&sm->afull[(aa + 1) % STC_ASLOTS]));
          }
        }
        a += STC_NTILE;
      }
    }
  } else {
    // ---------------- epilogue ----------------
    const int q4 = warp & 3;
    const int row = 32 * q4 + lane;
    const int twoK = 2 * K;
    const int mi = row / twoK, rem = row - mi * twoK, k = rem >> 1, ri = rem & 1;
    unsigned ul = 0;
    for (int u = blockIdx.x; u < pl.nunits && ok; u += gridDim.x, ++ul) {
      int m, part, g;
      unit(u, m, part, g);
      const int e = g * pl.G + mi;
      const bool live = (mi < pl.G) && (e < E);
      const int b = ul % pl.nacc;
      ok = warp_wait(smem_addr(&sm->accfull[b]), (ul / pl.nacc) & 1u, err, ATC_ERR);
      if (!ok) break;
      tc_fence_after();
      const unsigned tl = tbase + ((unsigned)(32 * q4) << 16) + (unsigned)(b * STC_NREG * JT);
      // sf[e][m][j][k][6] complex: the thread with ri = 0 writes fields 0..2,
      // its partner (ri = 1) fields 3..5 of level k, each as three (Re, Im)
      float* sfe = reinterpret_cast<float*>(d.sf) +
                   ((((size_t)e * M + m) * J + part * JT) * K + k) * 12 + ri * 6;
      for (int c0 = 0; c0 < JT; c0 += 8) {
        float v[STC_NREG][8];
#pragma unroll
        for (int r = 0; r < STC_NREG; ++r) tmem_ld8(tl + (unsigned)(r * JT + c0), v[r]);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          float o[6];
#pragma unroll
          for (int x = 0; x < 3; ++x) {
            // the partner's half: ri = 0 sends fields 3..5, ri = 1 fields 0..2
            const float send = ri ? v[x][i] : v[3 + x][i];
            const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
            const float mine = ri ? v[3 + x][i] : v[x][i];
            o[2 * x] = ri ? recv : mine;          // Re of field (ri ? 3 : 0) + x
            o[2 * x + 1] = ri ? mine : recv;      // Im
          }
          if (live) {
            float* dst = sfe + (size_t)(c0 + i) * K * 12;
            *reinterpret_cast<float2*>(dst) = make_float2(o[0], o[1]);
            *reinterpret_cast<float2*>(dst + 2) = make_float2(o[2], o[3]);
            *reinterpret_cast<float2*>(dst + 4) = make_float2(o[4], o[5]);
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
