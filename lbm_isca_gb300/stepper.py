"""Host driver of the fused ensemble stepper (lbm_stepper_* in the C ABI).

The stepper owns the packed spectral state of E members and every operator
the four step kernels read, in the working precision (FP64 or FP32).  Setup
quantities (Legendre tables, Gauss weights, semi-implicit inverses) are
produced in FP64 by the library's setup kernels and rounded once.

Step bookkeeping follows model.py:213-247: a step carries its dt (the
start-up calls use delt/2^(inistp-istep+1)), whether the previous level is
set by copy (forward start) or by the Robert-Asselin filter, and how the
grid ps of the previous level is brought up to date (the ps part of the
filter is applied at the top of the next step, once ps(t+dt) exists in grid
space).  Runs of identical steady-state steps are captured once into a CUDA
graph (lbm_graph_capture) and replayed.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from . import ops as _ops
from ._lib import StepCtl, StepperDesc, check, lib, ptr
from .backend import stream_handle
from .constants import EPSVT, KAPPA, RAIR

VERT_ROWS = 12   # LBM_VERT_COUNT in include/lbm_gb300.h


def tc_anal_image(P, H, nn1a, N):
    """Table image of the tensor-core Legendre analysis (the tc_anal layout of
    include/lbm_gb300.h): per m, per step of 16 latitudes, the tables P, H
    and nn1a P over rows n = m..N padded to a multiple of 16, each split from
    FP64 into three bfloat16 pieces (b0 = bf16(x), b1 = bf16(x - b0),
    b2 = bf16(x - b0 - b1)), each piece one K-major tile of 8-row x 16-byte
    core matrices.  P, H: [M][M][J] FP64 (any device); returns int16 words."""
    J = P.shape[-1]
    KS = J // 16
    P = P.to(torch.float64)
    tabs = (P, H.to(torch.float64), P * nn1a.to(torch.float64)[None, :, None])
    out = []
    for m in range(N + 1):
        nr = N + 1 - m
        nb = (nr + 15) // 16 * 16
        T = torch.zeros((3, nb, J), device=P.device, dtype=torch.float64)
        for t in range(3):
            T[t, :nr] = tabs[t][m, m:, :]
        pieces, r = [], T
        for _ in range(3):
            b = r.to(torch.bfloat16)
            pieces.append(b.view(torch.int16))
            r = r - b.to(torch.float64)
        x = torch.stack(pieces, 1)                        # [t][p][nb][J]
        x = x.reshape(3, 3, nb // 8, 8, KS, 2, 8)          # [t][p][rg][r8][s][kc][k8]
        out.append(x.permute(4, 0, 1, 2, 5, 3, 6).reshape(-1))
    return torch.cat(out).contiguous()


def tc_synth_image(P, H, invlap, N):
    """Table image of the tensor-core Legendre synthesis (the tc_synth layout
    of include/lbm_gb300.h): per m, per latitude part (JT = J latitudes, or
    J / 2 when six regions of J columns exceed the tensor memory), per step
    of 16 rows n, the tables m P il, -H il, H il and P (il the inverse
    Laplacian factor of row n) as JT x 16 tiles (rows = latitudes, K = n),
    each split from FP64 into three bfloat16 pieces."""
    J = P.shape[-1]
    nparts = 1 if 6 * J <= 512 else 2
    JT = J // nparts
    P = P.to(torch.float64)
    H = H.to(torch.float64)
    il = invlap.to(torch.float64)
    out = []
    for m in range(N + 1):
        nr = N + 1 - m
        ks = (nr + 15) // 16
        Pm, Hm, ilm = P[m, m:, :], H[m, m:, :], il[m:, None]
        T = torch.zeros((4, ks * 16, J), device=P.device, dtype=torch.float64)
        T[0, :nr] = m * Pm * ilm
        T[1, :nr] = -Hm * ilm
        T[2, :nr] = Hm * ilm
        T[3, :nr] = Pm
        for part in range(nparts):
            X = T[:, :, part * JT:(part + 1) * JT].permute(0, 2, 1)     # [t][j][n]
            pieces, r = [], X
            for _ in range(3):
                b = r.to(torch.bfloat16)
                pieces.append(b.view(torch.int16))
                r = r - b.to(torch.float64)
            x = torch.stack(pieces, 1)                                # [t][p][JT][ks*16]
            x = x.reshape(4, 3, JT // 8, 8, ks, 2, 8)                  # [t][p][rg][r8][s][kc][k8]
            out.append(x.permute(4, 0, 1, 2, 5, 3, 6).reshape(-1))
    return torch.cat(out).contiguous()


def tc_dft_image(N, I, device="cpu"):
    """Table image of the longitude analysis on the tensor cores (the tc_dft
    layout of include/lbm_gb300.h): per step of 16 longitudes, the 128 x 16
    tile W[2m][i] = cos(2 pi m i / I) / I, W[2m + 1][i] = -sin(2 pi m i / I) /
    I (zero rows for m > N), split from FP64 into three bfloat16 pieces, each
    a K-major tile of 8-row x 16-byte core matrices; then the FP32 table
    cos(2 pi t / I), t < I, of the surface rows' FMA kernel.  Returns int16
    words."""
    KS = I // 16
    m = torch.arange(64, dtype=torch.float64, device=device)
    i = torch.arange(I, dtype=torch.float64, device=device)
    ang = (2.0 * np.pi / I) * torch.remainder(m[:, None] * i[None, :], I)
    W = torch.zeros((128, I), dtype=torch.float64, device=device)
    W[0::2] = torch.cos(ang) / I
    W[1::2] = -torch.sin(ang) / I
    W[2 * (N + 1):] = 0.0
    pieces, r = [], W
    for _ in range(3):
        b = r.to(torch.bfloat16)
        pieces.append(b.view(torch.int16))
        r = r - b.to(torch.float64)
    x = torch.stack(pieces, 0)                            # [p][128][I]
    x = x.reshape(3, 16, 8, KS, 2, 8)                     # [p][rg][r8][s][kc][k8]
    cs = torch.cos((2.0 * np.pi / I) * i).to(torch.float32).view(torch.int16)
    return torch.cat([x.permute(3, 0, 1, 4, 2, 5).reshape(-1), cs]).contiguous()


class EnsembleStepper:
    """Fused GPU time stepping of `nmem` members sharing one basic state."""

    #: precision -> products of the tensor-core contractions (0: FMA pipes)
    LEGENDRE = {"fp64": 0, "fp32": 0, "bf16x3": 6, "bf16split": 3}
    #: precision -> contractions kept on the FMA pipes by default (tc_off bits:
    #: 0 Legendre analysis, 1 Legendre synthesis, 2 longitude analysis).  The
    #: tensor cores' FP32 accumulation rounds toward zero; in bf16x3 only the
    #: longitude analysis of the level rows goes to them by default, which
    #: keeps the T42L20 day-30 error at 6.3e-6 (with the Legendre
    #: contractions there too it reaches 1.1e-5, over the 1e-5 FP32 gate).
    TC_OFF = {"bf16x3": 3, "bf16split": 0}

    def __init__(self, sp, vg, bst, damping, semi, vdiff, nmem, precision="fp64",
                 robert=0.04, strictly_linear=False, stream=None, tc_off=None):
        if precision not in self.LEGENDRE:
            raise ValueError(f"precision must be one of {sorted(self.LEGENDRE)}")
        self.sp, self.vg, self.bst = sp, vg, bst
        self.semi, self.vdiff = semi, vdiff
        self.dev = dev = sp.device
        self.precision = precision
        self.rd = torch.float64 if precision == "fp64" else torch.float32
        self.cd = torch.complex128 if precision == "fp64" else torch.complex64
        self.prec_id = _lib.LBM_F64 if precision == "fp64" else _lib.LBM_F32
        self.legendre = self.LEGENDRE[precision]
        # placement and tiles of the tensor-core kernels (autotune.tune()):
        # which contractions stay on the FMA kernels, members per MMA tile
        self.tc_off = int(self.TC_OFF.get(precision, 0) if tc_off is None else tc_off)
        self.tc_g = 0
        if not 0 <= self.tc_off <= 7:
            raise ValueError("tc_off must be in 0..7")
        self.E = E = int(nmem)
        self.N = N = sp.nmax
        self.M = M = N + 1
        self.J, self.I, self.K = J, I, K = sp.nlat, sp.nlon, vg.kmax
        self.NS = NS = M * (M + 1) // 2
        self.stream = stream if stream is not None else torch.cuda.Stream(device=dev)
        rd, cd = self.rd, self.cd
        mm, nn = np.nonzero(np.triu(np.ones((M, M), dtype=bool)))
        self.pm = torch.as_tensor(mm, device=dev)
        self.pn = torch.as_tensor(nn, device=dev)
        R = lambda x: x.to(device=dev, dtype=rd).contiguous()   # noqa: E731
        JH = J // 2
        self.symp = R(sp.pnm[self.pm, self.pn, :JH])
        self.symh = R(sp.hnm[self.pm, self.pn, :JH])
        self.tw = R(sp._tw64)
        # longitude DFT table of the FP32 grid kernel: (cos, sin)(2 pi m i/I), i <= I/4
        Q = I // 4
        ang = 2.0 * np.pi * np.outer(np.arange(M), np.arange(Q + 1)) / I
        self.dft = torch.as_tensor(np.stack([np.cos(ang), np.sin(ang)], -1),
                                   device=dev, dtype=torch.float32).contiguous()
        coslat = sp.coslat
        gwdel = torch.as_tensor(sp.gwdel, device=dev)
        self.jfac = R(torch.stack([torch.as_tensor(sp.gw, device=dev), gwdel * coslat,
                                   1.0 / (sp.a * coslat), coslat]))
        vh = vg.host
        vert = np.zeros((VERT_ROWS, K + 1))
        vert[0, :K] = vh("dsig")
        vert[1, :] = vh("sigm")
        vert[2, :K] = vh("alpha")
        vert[3, :K] = vh("w3")
        vert[4, :K] = vh("wP")
        vert[5, :K] = RAIR * vh("cpg")
        vert[6, :K] = RAIR * vh("dlog3")
        vert[7, :K] = RAIR * vh("alpha")
        vert[8, :K] = vh("tbar")
        vert[9, :K] = KAPPA * vh("tbar")
        vert[10, :K] = vh("sig")
        vert[11, :K] = vh("gg")
        self.vert = R(torch.as_tensor(vert))
        tref = torch.as_tensor(vh("tbar"), device=dev)
        b = bst
        def half_diff(x):          # 0.5 (x[k+1] - x[k]), 0 at the top level (FP64)
            h = torch.zeros_like(x)
            h[..., :-1] = 0.5 * (x[..., 1:] - x[..., :-1])
            return h
        f3 = [b.u, b.v, b.t, b.q, b.tv, b.absvor, b.div, b.x5, b.t - tref, b.tv - tref,
              half_diff(b.u), half_diff(b.v), half_diff(b.t), half_diff(b.q)]
        self.b3 = R(torch.stack([x.permute(0, 2, 1) for x in f3]))        # [14][J][K][I]
        self.bsd = R(b.sdot.permute(0, 2, 1))                             # [J][K+1][I]
        dsig = torch.as_tensor(vh("dsig"), device=dev)
        self.b2 = R(torch.stack([b.pix, b.piy, b.ps, (b.u * dsig).sum(-1),
                                 (b.v * dsig).sum(-1)]))                  # [5][J][I]
        self.lap = R(sp.laplace)
        self.invlap = R(sp.inv_laplace)
        self.nn1a = R(-sp.laplace)
        self.kv, self.kd = R(damping.kv), R(damping.kd)
        self.ktt, self.kq = R(damping.ktt), R(damping.kq)
        self.ww = R(torch.as_tensor(vh("ww")))
        self.tmtx = R(torch.as_tensor(vh("tmtx")))
        self.robert = float(robert)
        self.strictly_linear = int(bool(strictly_linear))
        self.vd_on = [int(vdiff.coef[n] is not None) for n in ("vor", "div", "t", "q")]
        # state and intermediates
        z = lambda *s: torch.zeros(s, device=dev, dtype=cd)   # noqa: E731
        self.sa3, self.sas, self.sb3 = z(E, 4, NS, K), z(E, 4, NS), z(E, 4, NS, K)
        self.psa = torch.zeros((E, J, I), device=dev, dtype=rd)
        self.psb = torch.zeros((E, J, I), device=dev, dtype=rd)
        self.sf, self.sfs = z(E, M, J, K, 6), z(E, M, J, 5)
        self.af, self.afs = z(E, M, J, K, 7), z(E, M, J, 2)
        self.tend, self.tends = z(E, 4, NS, K), z(E, 2, NS)
        self.tc_anal = self._tc_anal_image() if self.legendre else None
        self.tc_synth = (tc_synth_image(sp.pnm, sp.hnm, sp.inv_laplace, N)
                         if self.legendre else None)
        # the longitude analysis of the level rows on the tensor cores where
        # its plan applies (nlon <= 128, 9 kmax <= 256 rows)
        self.tc_dft = (tc_dft_image(N, I, dev) if self.legendre and I <= 128
                       and 9 * K <= 256 else None)
        # FP32 grid rows between the longitude transforms and the column algebra
        if precision != "fp64":
            f = lambda *s_: torch.zeros(s_, device=dev, dtype=torch.float32)   # noqa: E731
            self.grid6 = f(E, J, 6 + 6 * K, I)
            self.grid9 = f(E, J, 2 + 9 * K, I)
        else:
            self.grid6 = self.grid9 = None
        self.err = torch.zeros(1, device=dev, dtype=torch.int32)
        self.err_member = torch.zeros(E, device=dev, dtype=torch.int32)
        self.frc3 = self.frcs = None
        self.frc_shared = 1
        self._dts = []
        self.minv = self.vdm = None
        self._graphs = {}
        self.pending_ps_mode = 0
        self._desc = None
        self._oargs = None
        self._null = torch.empty(0, device=dev, dtype=torch.float32)

    def _tc_anal_image(self):
        sp = self.sp
        if self.J % 16:
            raise ValueError("the tensor-core analysis needs nlat a multiple of 16")
        return tc_anal_image(sp.pnm, sp.hnm, -sp.laplace, self.N)

    # ------------------------------------------------------------------
    def set_timesteps(self, dts):
        """Operator sets (semi-implicit inverse, vertical diffusion) per dt."""
        dts = [float(x) for x in dts]
        if dts == self._dts:
            return
        K, M = self.K, self.M
        mins, vds = [], []
        for dt in dts:
            _, minv, _ = self.semi.matrices(dt)
            mins.append(minv.transpose(1, 2))                    # stored (n, l, k)
            ops = self.vdiff.operators(dt)
            eye = torch.eye(K, device=self.dev, dtype=torch.float64)
            # stored as (operator - identity)^T: the kernel adds the small
            # correction to the value itself, keeping its relative precision
            vds.append(torch.stack([((ops[n] - eye) if ops[n] is not None else 0 * eye).T
                                    for n in ("vor", "div", "t", "q")]))
        self.minv = torch.stack(mins).to(self.rd).contiguous()   # [nsets][M][K][K]
        self.vdm = torch.stack(vds).to(self.rd).contiguous()     # [nsets][4][K][K]
        self._dts = dts
        self._drop_graphs()
        self._desc = None

    def set_index(self, dt):
        return self._dts.index(float(dt))

    def set_forcing(self, frc_vor=None, frc_div=None, frc_t=None, frc_pi=None, frc_q=None,
                    per_member=False):
        """Spectral forcings, rectangle layout ((E,) M, M, K) / ((E,) M, M)."""
        if all(x is None for x in (frc_vor, frc_div, frc_t, frc_pi, frc_q)):
            self.frc3 = self.frcs = None
            self.frc_shared = 1
            self._desc = None
            self._drop_graphs()
            return
        Ef = self.E if per_member else 1
        f3 = torch.zeros((Ef, 4, self.NS, self.K), device=self.dev, dtype=self.cd)
        fs = torch.zeros((Ef, self.NS), device=self.dev, dtype=self.cd)
        for i, x in enumerate((frc_vor, frc_div, frc_t, frc_q)):
            if x is not None:           # (B, M, M, K), B = 1 or E
                p = self.pack(x).reshape(-1, self.NS, self.K)
                f3[:, i] = p.expand(Ef, self.NS, self.K)
        if frc_pi is not None:          # (B, M, M)
            p = self.pack(frc_pi).reshape(-1, self.NS)
            fs[:] = p.expand(Ef, self.NS)
        new_ptrs = self.frc3 is None
        if self.frc3 is not None and self.frc3.shape == f3.shape:
            # in place, ordered after the steps already queued on the stepper's
            # stream (they may still read the old forcing)
            self.stream.wait_stream(torch.cuda.current_stream(self.dev))
            with torch.cuda.stream(self.stream):
                self.frc3.copy_(f3)
                self.frcs.copy_(fs)
            f3.record_stream(self.stream)
            fs.record_stream(self.stream)
        else:
            # new buffers: the stepper's stream must see them written
            self.stream.wait_stream(torch.cuda.current_stream(self.dev))
            self.frc3, self.frcs = f3, fs
            new_ptrs = True
        self.frc_shared = 0 if per_member else 1
        if new_ptrs:
            self._desc = None
            self._drop_graphs()

    # ------------------------------------------------------------------
    def pack(self, x):
        """(..., M, M[, K]) rectangle -> (..., NS[, K]) packed, working precision."""
        x = x.to(self.dev)
        if x.shape[-2:] == (self.M, self.M):
            return x[..., self.pm, self.pn].to(self.cd)
        return x[..., self.pm, self.pn, :].to(self.cd)

    def unpack(self, p, has_k=True):
        lead = p.shape[:-2] if has_k else p.shape[:-1]
        shape = lead + (self.M, self.M) + ((p.shape[-1],) if has_k else ())
        out = torch.zeros(shape, device=self.dev, dtype=torch.complex128)
        if has_k:
            out[..., self.pm, self.pn, :] = p.to(torch.complex128)
        else:
            out[..., self.pm, self.pn] = p.to(torch.complex128)
        return out

    def load(self, a_spec, b_spec, psa, psb):
        """Load the current level (spectral dict incl. pi), the previous level
        (spectral vor/div/t/q) and both grid ps' fields; member axis first."""
        for i, k in enumerate(("vor", "div", "t", "q")):
            self.sa3[:, i] = self.pack(a_spec[k]).reshape(self.E, self.NS, self.K)
            self.sb3[:, i] = self.pack(b_spec[k]).reshape(self.E, self.NS, self.K)
        self.sas[:, 0] = self.pack(a_spec["pi"]).reshape(self.E, self.NS)
        self.psa.copy_(psa.reshape(self.E, self.J, self.I))
        self.psb.copy_(psb.reshape(self.E, self.J, self.I))
        self.pending_ps_mode = 0
        self.err.zero_()
        self.err_member.zero_()
        with torch.cuda.stream(self.stream):
            torch.cuda.current_stream().wait_stream(torch.cuda.default_stream(self.dev))
            torch.ops.lbm_gb300.stepper_colsum(*self.op_args())
            torch.ops.lbm_gb300.stepper_prime(*self.op_args())

    def load_zero(self):
        """Load the zero state (both levels, both grid ps'): the same as
        load() of zero fields, without transforming them."""
        with torch.cuda.stream(self.stream):
            torch.cuda.current_stream().wait_stream(torch.cuda.default_stream(self.dev))
            for t in (self.sa3, self.sas, self.sb3, self.psa, self.psb, self.err,
                      self.err_member):
                t.zero_()
            self.pending_ps_mode = 0
            torch.ops.lbm_gb300.stepper_prime(*self.op_args())

    def op_args(self):
        """(state, work, operators, dims, consts) of the torch.ops.lbm_gb300
        stepper operators (lists in the orders of ops.STEP_*; an empty tensor
        stands for NULL)."""
        if self._desc is not None and self._oargs is not None:
            return self._oargs
        z = lambda t: self._null if t is None else t      # noqa: E731
        state = [getattr(self, n) for n in _ops.STEP_STATE]
        work = [z(getattr(self, n)) for n in _ops.STEP_WORK]
        names = {"vdiff": "vdm"}
        opsl = [z(getattr(self, names.get(n, n))) for n in _ops.STEP_OPS]
        dims = [self.prec_id, self.E, self.J, self.I, self.N, self.K, len(self._dts),
                self.strictly_linear] + list(self.vd_on) + [self.frc_shared, self.legendre,
                                                            self.tc_off, self.tc_g]
        consts = [KAPPA, EPSVT, self.robert]
        self.desc()
        self._oargs = (state, work, opsl, dims, consts)
        return self._oargs

    def desc(self):
        if self._desc is not None:
            return self._desc
        self._oargs = None
        self.desc_gen = getattr(self, "desc_gen", 0) + 1     # counts rebuilt descriptors
        d = StepperDesc()
        d.prec = self.prec_id
        d.nmem, d.nlat, d.nlon, d.nmax, d.kmax = self.E, self.J, self.I, self.N, self.K
        d.nsets = len(self._dts)
        d.strictly_linear = self.strictly_linear
        for i in range(4):
            d.vd_on[i] = self.vd_on[i]
        d.frc_shared = self.frc_shared
        d.kappa, d.epsvt, d.robert = KAPPA, EPSVT, self.robert
        for name in ("symp", "symh", "tw", "jfac", "vert", "b3", "bsd", "b2", "lap", "invlap",
                     "nn1a", "kv", "kd", "ktt", "kq", "ww", "tmtx", "sa3", "sas", "sb3", "psa",
                     "psb", "sf", "sfs", "af", "afs", "tend", "tends", "grid6", "grid9"):
            setattr(d, name, ptr(getattr(self, name)))
        d.minv = ptr(self.minv)
        d.vdiff = ptr(self.vdm)
        d.frc3 = ptr(self.frc3)
        d.frcs = ptr(self.frcs)
        d.dft = ptr(self.dft)
        d.err = C.cast(C.c_void_p(self.err.data_ptr()), C.POINTER(C.c_int))
        d.err_member = C.cast(C.c_void_p(self.err_member.data_ptr()), C.POINTER(C.c_int))
        d.legendre = self.legendre
        d.tc_anal = ptr(self.tc_anal)
        d.tc_synth = ptr(self.tc_synth)
        d.tc_dft = ptr(self.tc_dft)
        d.tc_off, d.tc_g = self.tc_off, self.tc_g
        self._desc = d
        return d

    # ------------------------------------------------------------------
    def _ctl(self, steps):
        arr = (StepCtl * len(steps))()
        for i, (dt, start, psm) in enumerate(steps):
            arr[i].dt = float(dt)
            arr[i].set = self.set_index(dt)
            arr[i].ps_mode = psm
            arr[i].ra_mode = 0 if start else 1
        return arr

    def plan(self, steps):
        """[(dt, start)] -> [(dt, start, ps_mode)] continuing from the current
        pending ps update."""
        out = []
        pend = self.pending_ps_mode
        for dt, start in steps:
            out.append((dt, start, pend))
            pend = 1 if start else 2
        return out, pend

    def run(self, steps, use_graph=True, graph_chunk=72):
        """Advance through `steps` = [(dt, is_start_step), ...]."""
        planned, pend = self.plan(steps)
        s = stream_handle(self.stream)
        L = lib()
        self.stream.wait_stream(torch.cuda.default_stream(self.dev))
        with torch.cuda.stream(self.stream):
            d = self.desc()
            i = 0
            while i < len(planned):
                dt, start, psm = planned[i]
                steady = (not start) and psm == 2
                j = i
                while j < len(planned) and planned[j] == planned[i]:
                    j += 1
                n_same = j - i
                if use_graph and steady and n_same >= 2:
                    n = min(n_same, graph_chunk)
                    g = self._graph(planned[i:i + n])
                    check(L.lbm_graph_launch(g, s), "lbm_graph_launch")
                    i += n
                else:
                    torch.ops.lbm_gb300.stepper_run(*self.op_args(), [float(dt)],
                                                    [self.set_index(dt)], [int(psm)],
                                                    [0 if start else 1])
                    i += 1
        self.pending_ps_mode = pend

    def _graph(self, planned):
        key = (len(planned),) + planned[0]
        g = self._graphs.get(key)
        if g is None:
            ctl = self._ctl(planned)
            h = C.c_void_p()
            check(lib().lbm_graph_capture(C.byref(self.desc()), ctl, len(planned),
                                          stream_handle(self.stream), C.byref(h)),
                  "lbm_graph_capture")
            g = h
            self._graphs[key] = g
        return g

    def _drop_graphs(self):
        for g in self._graphs.values():
            lib().lbm_graph_destroy(g)
        self._graphs = {}

    def flush(self):
        """Bring psa/psb up to date with the last step."""
        if self.pending_ps_mode == 0:
            return
        self.stream.wait_stream(torch.cuda.default_stream(self.dev))
        with torch.cuda.stream(self.stream):
            torch.ops.lbm_gb300.stepper_flush(*self.op_args(), int(self.pending_ps_mode))
        self.pending_ps_mode = 0

    # ---- daily history (model.py:257-277) ---------------------------------
    def hist_begin(self):
        """FP64 accumulators and previous-sample copies of the spectral state
        (sa3, sas) and the grid ps' (psa) for the daily history means."""
        self._hist = {}
        for name in ("sa3", "sas", "psa"):
            cur = getattr(self, name)
            n = cur.numel() * (2 if cur.is_complex() else 1)
            self._hist[name] = (torch.zeros_like(cur),
                                torch.zeros(n, device=self.dev, dtype=torch.float64))
        self.hist_n = 0

    def hist_sample(self, what, mode):
        """Accumulate the top-of-step sample: what = "spec" (state, before the
        step's kernels) or "ps" (grid ps', after them); mode 0 only records
        the sample (start-up steps), mode 1 adds 0.5 (cur + previous)."""
        names = ("sa3", "sas") if what == "spec" else ("psa",)
        with torch.cuda.stream(self.stream):
            for name in names:
                cur = getattr(self, name)
                prev, acc = self._hist[name]
                torch.ops.lbm_gb300.history_accumulate(cur, prev, acc, 0.5, int(mode))
        if what == "ps" and mode == 1:
            self.hist_n += 1

    def hist_reset(self):
        self.stream.wait_stream(torch.cuda.default_stream(self.dev))
        with torch.cuda.stream(self.stream):
            for _, acc in self._hist.values():
                acc.zero_()
        self.hist_n = 0

    def hist_mean(self):
        """Mean spectral state (rectangle complex128 dict incl. pi, member axis
        first) and mean grid ps' [E][J][I] of the accumulated samples."""
        torch.cuda.default_stream(self.dev).wait_stream(self.stream)
        n = max(self.hist_n, 1)
        E, NS, K = self.E, self.NS, self.K
        a3 = torch.view_as_complex(self._hist["sa3"][1].view(E, 4, NS, K, 2)) / n
        as_ = torch.view_as_complex(self._hist["sas"][1].view(E, 4, NS, 2)) / n
        spec = {k: self.unpack(a3[:, i]) for i, k in enumerate(("vor", "div", "t", "q"))}
        spec["pi"] = self.unpack(as_[:, 0], has_k=False)
        ps = self._hist["psa"][1].view(E, self.J, self.I) / n
        return spec, ps

    def launches_per_step(self):
        """Kernel launches of one step (lbm_stepper_run): FP64 k_grid,
        k_anal, k_implicit, k_synth; FP32 k_idft, k_alg, k_fdft, k_anal,
        k_implicit, k_synth, where each contraction on the tensor cores is
        two launches (the tensor-core kernel and the surface fields' FMA
        kernel)."""
        if self.precision == "fp64":
            return 4
        n = 6
        if self.legendre:
            n += int(not (self.tc_off & 1)) + int(not (self.tc_off & 2))
            n += int(self.tc_dft is not None and not (self.tc_off & 4))
        return n

    def check_finite(self):
        """False when a member produced a non-finite value (bit 0 of err);
        raises if a tensor-core kernel gave up a bounded wait (bit 1)."""
        self.stream.synchronize()
        e = int(self.err.item())
        if e & 2:
            raise RuntimeError("lbm_gb300: a tensor-core kernel timed out waiting for its "
                               "pipeline (results of this run are invalid)")
        return (e & 1) == 0

    def bad_members(self):
        """Indices of the members that produced a non-finite value since the
        state was loaded (the per-member flags k_implicit sets)."""
        self.stream.synchronize()
        return torch.nonzero(self.err_member).flatten().tolist()

    def grid_level(self, level):
        """Grid u, v, T, q ([E][J][I][K], FP64) of the current level ("a") or
        of the filtered previous level ("b"), from the stepper's own FP32
        synthesis kernels (Legendre synthesis into sf, then the longitude
        synthesis into grid6) -- FP32 state only.  Synthesising "a" leaves
        sf as priming left it, so "b" is taken first when both are wanted."""
        if self.precision == "fp64":
            raise ValueError("grid_level needs an FP32-state stepper")
        d = StepperDesc.from_buffer_copy(self.desc())
        if level == "b":
            d.sa3 = ptr(self.sb3)
        ctl = self._ctl([(self._dts[0], False, 0)])
        s = stream_handle(self.stream)
        E, J, I, K = self.E, self.J, self.I, self.K
        self.stream.wait_stream(torch.cuda.default_stream(self.dev))
        with torch.cuda.stream(self.stream):
            for kern in (3, 4):          # Legendre synthesis, longitude synthesis
                check(lib().lbm_stepper_launch(C.byref(d), ctl, kern, s),
                      "lbm_stepper_launch")
            rows = self.grid6.view(E, J, 6 + 6 * K, I)[:, :, 6:].view(E, J, K, 6, I)
            out = {}
            for f, name in ((0, "u"), (1, "v"), (4, "t"), (5, "q")):
                t = torch.empty((E, J, I, K), device=self.dev, dtype=torch.float64)
                t.copy_(rows[:, :, :, f, :].permute(0, 1, 3, 2))
                out[name] = t
        torch.cuda.default_stream(self.dev).wait_stream(self.stream)
        return out

    def snapshot(self):
        """Copy of the current level (rectangle dict incl. pi)."""
        torch.cuda.default_stream(self.dev).wait_stream(self.stream)
        a = {k: self.unpack(self.sa3[:, i]) for i, k in enumerate(("vor", "div", "t", "q"))}
        a["pi"] = self.unpack(self.sas[:, 0], has_k=False)
        return a

    def spectral_state(self):
        """Current (a) and previous (b) levels as rectangle dicts (complex128)."""
        torch.cuda.default_stream(self.dev).wait_stream(self.stream)
        a, b = {}, {}
        for i, k in enumerate(("vor", "div", "t", "q")):
            a[k] = self.unpack(self.sa3[:, i])
            b[k] = self.unpack(self.sb3[:, i])
        a["pi"] = self.unpack(self.sas[:, 0], has_k=False)
        return a, b

    def __del__(self):
        try:
            self._drop_graphs()
        except Exception:
            pass
