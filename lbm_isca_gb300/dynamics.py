"""Linearised primitive-equation tendencies (drop-in for pylbm_isca/dynamics.py).

``Dynamics.tendencies`` keeps the reference's signature and return value
(five spectral tendencies, dynamics.py:156-271).  The transforms are the
lbm_gb300 transform kernels and the whole grid-point part -- column sums,
sigma-dot, virtual temperature, Simmons-Burridge omega factor, adiabatic and
advection terms, pressure gradient, vertical advection, hydrostatic and
energy-conversion operators, kinetic energy, omega diagnostic -- is one
fused launch of ``lbm_tendency_grid``.  The fused ensemble stepper runs the
same algebra inside its own grid kernel; this class is the reference-layout
entry point (used directly by callers and for a forward start from an
arbitrary grid state).
"""

from __future__ import annotations

import numpy as np
import torch

from . import ops as _ops
from .backend import to_device
from .constants import EPSVT, KAPPA, OMEGA, RAIR


def _column_sum(x, dsig):
    """S[k] = sum_{l>=k} dsig_l x_l, trailing zero (dynamics.py:96-102)."""
    w = x * dsig
    out = torch.zeros(x.shape[:-1] + (x.shape[-1] + 1,), dtype=x.dtype, device=x.device)
    out[..., :-1] = torch.flip(torch.cumsum(torch.flip(w, (-1,)), -1), (-1,))
    return out


def _sigma_dot(ssum, sigm):
    """dynamics.py:105-114."""
    sd = sigm * ssum[..., :1] - ssum
    sd[..., 0] = 0.0
    sd[..., -1] = 0.0
    return sd


def _vert_advect(field, sdot, dsig):
    """dynamics.py:117-143 (used for the time-constant basic state only)."""
    K = field.shape[-1]
    lead = torch.broadcast_shapes(field.shape[:-1], sdot.shape[:-1])
    flux = torch.zeros(lead + (K + 1,), dtype=field.dtype, device=field.device)
    flux[..., 1:K] = sdot[..., 1:K] * 0.5 * (field[..., 1:K] + field[..., :K - 1])
    dsdot = sdot[..., 1:] - sdot[..., :-1]
    return (flux[..., 1:] - flux[..., :-1] - field * dsdot) / dsig


class BasicStateTerms:
    """Basic-state derived fields (dynamics.py:51-93); one-off setup."""

    def __init__(self, sp, vgrid, bs):
        self.sp, self.vg = sp, vgrid
        dev = sp.device
        self.xp = torch
        self.u = to_device(bs.u, dev)
        self.v = to_device(bs.v, dev)
        self.t = to_device(bs.t, dev)
        self.q = to_device(bs.q, dev)
        self.ps = to_device(bs.ps, dev)
        self.coriol = torch.as_tensor((2.0 * OMEGA * sp.mu)[:, None], device=dev)
        self.vor, self.div_s = sp.uv_to_vordiv(self.u, self.v)
        self.vor_g = sp.wave_to_grid(self.vor)
        self.div = sp.wave_to_grid(self.div_s)
        self.lnps = torch.log(self.ps)
        self.pix, self.piy = sp.hgrad(sp.grid_to_wave(self.lnps))
        self.tv = self.t * (1.0 + EPSVT * self.q)
        self.padv = self.u * self.pix[..., None] + self.v * self.piy[..., None]
        self.ssum = _column_sum(self.div + self.padv, vgrid.dsig)
        self.sdot = _sigma_dot(self.ssum, vgrid.sigm)
        self.x5 = (vgrid.w3 * self.ssum[..., 1:] + vgrid.alpha * self.div
                   + vgrid.wP * self.padv)
        from .vertical import compute_tbar
        vgrid.set_reference_temperature(compute_tbar(self.tv))
        self.absvor = (self.vor_g + self.coriol[..., None]).contiguous()


class Dynamics:
    """Explicit (non-gravity-wave) tendencies (dynamics.py:146-271)."""

    def __init__(self, sp, vgrid, bst, strictly_linear=False):
        self.sp, self.vg, self.bs = sp, vgrid, bst
        self.strictly_linear = bool(strictly_linear)
        self.diag = {}

    def _grid_kernel(self, st, vor, div, pix, piy, frc_t, frc_ps, frc_q, want_omega=True,
                     lin=None):
        """One launch of lbm_tendency_grid.  ``lin = (u0, v0)`` selects the
        tangent-linear kinetic energy u0 u + v0 v in place of 0.5 (u^2 + v^2)."""
        sp, vg, bs = self.sp, self.vg, self.bs
        dev = sp.device
        u = st.u
        batched = u.dim() == 4
        E = u.shape[0] if batched else 1
        J, I, K = sp.nlat, sp.nlon, vg.kmax
        shp3 = tuple(u.shape)
        shp2 = shp3[:-1]

        def frc(x, full_shape):
            if x is None:
                return None, 0
            t = to_device(x, dev, u.dtype)
            per = int(np.prod(full_shape[1:])) if batched else 0
            stride = per if (batched and t.dim() == len(full_shape)) else 0
            return t, stride

        ft, ft_s = frc(frc_t, shp3)
        fp, fp_s = frc(frc_ps, shp2)
        fq, fq_s = frc(frc_q, shp3)
        named = {"dsig": vg.dsig, "sigm": vg.sigm, "alpha": vg.alpha, "w3": vg.w3, "wP": vg.wP,
                 "cpg": vg.cpg, "sig": vg.sig, "ww": vg.ww, "tmtx": vg.tmtx, "tref": vg.tbar,
                 "ub": bs.u, "vb": bs.v, "tb": bs.t, "qb": bs.q, "tvb": bs.tv,
                 "absvor": bs.absvor, "divb": bs.div, "x5b": bs.x5, "sdotb": bs.sdot,
                 "pixb": bs.pix, "piyb": bs.piy, "psb": bs.ps, "u": u, "v": st.v, "t": st.t,
                 "q": st.q, "vor": vor, "div": div, "pix": pix, "piy": piy, "ps": st.ps,
                 "frc_t": ft, "frc_ps": fp, "frc_q": fq,
                 "lin_u": None if lin is None else lin[0],
                 "lin_v": None if lin is None else lin[1]}
        outs = torch.ops.lbm_gb300.tendency_grid(
            [named[k] for k in _ops.TEND_INPUTS], E, J, I, K, int(self.strictly_linear),
            [KAPPA, EPSVT, RAIR], [ft_s, fp_s, fq_s], bool(want_omega))
        out = dict(zip(_ops.TEND_OUTPUTS, outs))
        if not want_omega:
            out["omega"] = None
        return out

    def tendencies(self, st, frc_t=None, frc_vor=None, frc_div=None, frc_ps=None,
                   frc_q=None):
        """Explicit tendencies of (vor, div, T, pi, q) in spectral space."""
        sp = self.sp
        vor_s, div_s = sp.uv_to_vordiv(st.u, st.v)
        vor = sp.wave_to_grid(vor_s)
        div = sp.wave_to_grid(div_s)
        pi = st.lnps_pert()
        pix, piy = sp.hgrad(sp.grid_to_wave(pi))
        o = self._grid_kernel(st, vor, div, pix, piy, frc_t, frc_ps, frc_q)
        wt_pi = sp.grid_to_wave(o["gt_pi"])
        wt_t = sp.neg_divergence(o["xu"], o["xv"]) + sp.grid_to_wave(o["gt"])
        wt_vor, wt_div = sp.uv_to_vordiv(o["fu"], o["fv"])
        wt_div = wt_div - sp.laplacian(sp.grid_to_wave(o["ke"]))
        if frc_vor is not None:
            wt_vor = wt_vor + sp.grid_to_wave(frc_vor)
        if frc_div is not None:
            wt_div = wt_div + sp.grid_to_wave(frc_div)
        wt_q = sp.neg_divergence(o["yu"], o["yv"]) + sp.grid_to_wave(o["g"])
        self.diag = {"vor": vor, "div": div, "vor_s": vor_s, "div_s": div_s,
                     "omega": o["omega"], "sdot": o["sdot"], "pi": pi}
        return wt_vor, wt_div, wt_t, wt_pi, wt_q
