"""Hand-written adjoint of the time step, with binomial checkpointing.

The reference has no adjoint.  This module differentiates the reference's
own step sequence (model.py:232-243):

    tend = Dynamics.tendencies(ga, frc_t)         (dynamics.py:156-271)
    prev = gb.to_spectral()                       (state.py:86-92)
    new  = Integrator.step(dt, prev, tend)        (integrator.py:264-315)
    gc   = load_spectral(new)                     (state.py:94-99)
    gb'  = ga (start) | RA(gb, ga, gc)            (state.py:110-128)
    ga'  = gc

It is linear about the basic state except the kinetic energy
0.5 (u^2 + v^2) of the tendency and the exact pi' <-> ps' conversions
(pi' = ln(ps_bar + ps') - ln(ps_bar), ps' = ps_bar (e^pi' - 1)); those are
linearised about the stored trajectory.

Pieces, all on the device:
* ``AdjointTransforms``: the transpose of every spectral operator of the
  step.  Each is the library's opposite transform with rescaled tables:
  the transpose of the inverse longitude transform is c_m I times the
  forward one (c_0 = 1, c_m = 2), the transpose of the forward one is
  h_m / I times the inverse one (h_0 = 1, h_m = 1/2), and the transpose of
  a Legendre contraction with i m is the other contraction with -i m.
* ``lbm_tendency_grid_adjoint`` / ``lbm_implicit_step_adjoint``: the grid
  columns and the spectral coefficients (adjoint.cu).
* ``TimeStep``: the step, its tangent-linear model and its adjoint, on grid
  states (``State``), functional (inputs are never modified).
* ``ForcingGradient``: the gradient of a scalar response of the final state
  with respect to a steady 3-D heating (the ``frc_t`` argument), by a
  forward sweep that stores at most ``snaps`` states on a binomial
  schedule (``checkpoint.schedule``) and a reverse sweep that re-advances
  from them.  ``HeatingResponse`` wraps it as a ``torch.autograd.Function``.
"""

from __future__ import annotations

import types

import numpy as np
import torch

from . import ops as _ops
from .backend import to_device
from .checkpoint import schedule as binomial_schedule
from .configs import response_box
from .constants import EPSVT, KAPPA, RAIR
from .dynamics import Dynamics
from .state import State

FIELDS = ("u", "v", "t", "q", "ps")


def _zeros_like_state(st):
    return types.SimpleNamespace(**{k: torch.zeros_like(getattr(st, k)) for k in FIELDS})


def _ns(**kw):
    return types.SimpleNamespace(**kw)


def _cat(xs, nd=3):
    """Concatenate fields along their last (level) axis; a field of fewer
    than ``nd`` dimensions (a surface field) counts as one level.  Transforms
    act column by column, so one launch over the concatenation gives each
    field exactly what its own launch would."""
    return torch.cat([x if x.dim() == nd else x.unsqueeze(-1) for x in xs], dim=-1)


def state_dot(a, b):
    """Euclidean inner product of two grid states (u v t q ps)."""
    return sum(float((getattr(a, k) * getattr(b, k)).sum()) for k in FIELDS)


def spec_dot(a, b):
    """Real inner product of complex spectral arrays: sum Re(conj(a) b)."""
    return float((a.conj() * b).real.sum())


# ---------------------------------------------------------------------------
# Transposed spectral operators
# ---------------------------------------------------------------------------
class AdjointTransforms:
    """Transposes of the operators of ``Spectral`` (spectral.py:159-276)
    under the Euclidean inner products of grid values and of (Re, Im)
    spectral coefficients."""

    def __init__(self, sp):
        if sp.precision not in ("fp64", "fp32"):
            raise ValueError("the adjoint runs in FP64 or FP32")
        self.sp = sp
        M, I = sp.nmax + 1, sp.nlon
        dev, rd = sp.device, sp.rdtype
        cm = torch.full((M,), 2.0 * I, dtype=torch.float64, device=dev)
        cm[0] = float(I)
        hm = torch.full((M,), 0.5 / I, dtype=torch.float64, device=dev)
        hm[0] = 1.0 / I
        # rescaled from the FP64 tables, rounded once to the working precision
        sc = lambda T, f: (T * f[:, None, None]).to(rd).contiguous()   # noqa: E731
        self.Pc = sc(sp.pnm, cm)
        self.Hc = sc(sp.hnm, cm)
        self.Pgw_h = sc(sp.pnm_gw, hm)
        self.Pgwdel_h = sc(sp.pnm_gwdel, hm)
        self.Hgwdel_h = sc(sp.hnm_gwdel, hm)
        self.neg_one = -torch.ones(M, dtype=rd, device=dev)
        self.neg_invlap = (-sp.inv_laplace).to(rd).contiguous()
        self.neg_cos = (-sp.coslat).to(rd).contiguous()

    def wave_to_grid_T(self, g):
        sp = self.sp
        g4, meta = sp._grid(g)
        return sp._ret_spec(sp._anal(sp._fwd(g4), self.Pc, 0), meta)

    def grid_to_wave_T(self, s):
        sp = self.sp
        s4, meta = sp._spec(s)
        return sp._ret_grid(sp._inv(sp._synth(s4, self.Pgw_h, 0)), meta)

    def hgrad_T(self, gx, gy):
        sp = self.sp
        x4, meta = sp._grid(gx)
        y4, _ = sp._grid(gy)
        rc = sp._t["rcos"]
        s = sp._anal(sp._fwd(x4, rc), self.Pc, 1, sp._fwd(y4, rc), self.Hc, 0, -1.0,
                     nfac=self.neg_one)
        return sp._ret_spec(s, meta)

    def uv_to_vordiv_T(self, vor, div):
        sp = self.sp
        v4, meta = sp._spec(vor)
        d4, _ = sp._spec(div)
        fv = sp._synth(v4, self.Pgwdel_h, 1, None, d4, self.Hgwdel_h, 0, None, 1.0)
        fu = sp._synth(d4, self.Pgwdel_h, 1, None, v4, self.Hgwdel_h, 0, None, -1.0)
        nc = self.neg_cos
        return sp._ret_grid(sp._inv(fu, nc), meta), sp._ret_grid(sp._inv(fv, nc), meta)

    def neg_divergence_T(self, s):
        sp = self.sp
        s4, meta = sp._spec(s)
        c = sp._t["cos"]
        fx = sp._inv(sp._synth(s4, self.Pgwdel_h, 1), c)
        fy = sp._inv(sp._synth(s4, self.Hgwdel_h, 0), c)
        return sp._ret_grid(fx, meta), sp._ret_grid(fy, meta)

    def vordiv_to_uv_T(self, u, v):
        sp = self.sp
        u4, meta = sp._grid(u)
        v4, _ = sp._grid(v)
        rc = sp._t["rcos"]
        fu, fv = sp._fwd(u4, rc), sp._fwd(v4, rc)
        nil = self.neg_invlap
        div = sp._anal(fu, self.Pc, 1, fv, self.Hc, 0, -1.0, nfac=nil)
        vor = sp._anal(fv, self.Pc, 1, fu, self.Hc, 0, 1.0, nfac=nil)
        return sp._ret_spec(vor, meta), sp._ret_spec(div, meta)


# ---------------------------------------------------------------------------
# The time step, its tangent-linear model and its adjoint
# ---------------------------------------------------------------------------
VG_FIELDS = ("dsig", "sigm", "alpha", "w3", "wP", "cpg", "sig", "ww", "tmtx", "tbar", "gg")
BS_FIELDS = ("u", "v", "t", "q", "tv", "absvor", "div", "x5", "sdot", "pix", "piy", "ps")


def _cast(obj, names, dtype, **extra):
    """A namespace of ``obj``'s named device arrays rounded to ``dtype``."""
    return types.SimpleNamespace(**{n: getattr(obj, n).to(dtype).contiguous() for n in names},
                                 **extra)


class TimeStep:
    """One reference step on grid states of an ``LBM``: one member, or E
    members (a batched model, ``make_ensemble_model``) whose states carry a
    leading member axis and advance together; members share the basic state
    and operators and are otherwise independent.

    ``precision="fp64"`` runs on the model's own FP64 objects.  ``"fp32"``
    runs the same kernels in FP32 (every C entry point of the step and its
    adjoint has an FP32 form): the transform tables come from an FP32
    ``Spectral`` of the same grid, and the vertical operators, basic state
    and semi-implicit / vertical-diffusion inverses are the model's FP64
    arrays rounded once."""

    def __init__(self, model, precision="fp64"):
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.m = model
        self.precision = precision
        self.nmem = model.nmem if model.batched else 1
        self.nd = 4 if model.batched else 3     # dimensions of a level-carrying field
        self.rd = torch.float64 if precision == "fp64" else torch.float32
        self.cd = torch.complex128 if precision == "fp64" else torch.complex64
        sp = model.sp
        if precision == "fp64":
            self.sp, self.vg, self.bs, self.dyn = sp, model.vg, model.bst, model.dyn
        else:
            self.sp = type(sp)(nlon=sp.nlon, nlat=sp.nlat, nmax=sp.nmax, radius=sp.a,
                               device=sp.device, precision="fp32")
            self.vg = _cast(model.vg, VG_FIELDS, self.rd, kmax=model.vg.kmax,
                            device=model.vg.device)
            self.bs = _cast(model.bst, BS_FIELDS, self.rd)
            self.dyn = Dynamics(self.sp, self.vg, self.bs, model.dyn.strictly_linear)
        self._iops = {}
        self.tr = AdjointTransforms(self.sp)
        self.ps_bar = model.ga.ps_bar.to(self.rd)
        self.lnps_bar = model.ga.lnps_bar.to(self.rd)
        self.gamma = float(model.cfg.robert)
        self.linear = bool(model.cfg.strictly_linear)

    # ---- helpers ------------------------------------------------------------
    def resources(self):
        """Every device tensor of the model the step reads (tables, basic
        state, operators, matrices).  A captured CUDA graph holds these so
        that its baked-in pointers stay valid even if the model replaces an
        attribute later (a second LBM on the same VerticalGrid resets its
        reference-temperature operators)."""
        m = self.m
        objs = [self.sp, self.sp._t, self.vg, self.bs, m.bst, m.damping, m.integ.semi,
                m.integ.semi._cache, m.integ.vdiff.minv, m.integ.vdiff._cache, self.tr,
                self._iops, {"ps_bar": self.ps_bar, "lnps_bar": self.lnps_bar}]
        out, seen = [], set()

        def grab(x, depth):
            if isinstance(x, torch.Tensor):
                if id(x) not in seen:
                    seen.add(id(x))
                    out.append(x)
            elif depth > 0 and isinstance(x, (dict, list, tuple)):
                for v in (x.values() if isinstance(x, dict) else x):
                    grab(v, depth - 1)

        for o in objs:
            grab(o if isinstance(o, dict) else vars(o), 3)
        return out

    def _state(self, u, v, t, q, ps):
        st = State.__new__(State)           # fields given: skip the constructor's setup
        st.xp, st.device = torch, self.sp.device
        st.ps_bar, st.lnps_bar = self.ps_bar, self.lnps_bar
        st.u, st.v, st.t, st.q, st.ps = u, v, t, q, ps
        return st

    def _lead(self):
        return (self.nmem,) if self.nd == 4 else ()

    def zero_state(self):
        J, I, K = self.sp.nlat, self.sp.nlon, self.vg.kmax
        f = dict(dtype=self.rd, device=self.sp.device)
        z3 = lambda: torch.zeros(self._lead() + (J, I, K), **f)   # noqa: E731
        return self._state(z3(), z3(), z3(), z3(), torch.zeros(self._lead() + (J, I), **f))

    def _pi(self, st):
        """pi' of a grid state.  FP64 keeps the reference's ln(ps_bar + ps') -
        ln(ps_bar) (state.py:77-79); FP32 takes log1p(ps' / ps_bar), the same
        quantity without the cancellation of two logarithms near 11.5."""
        if self.precision == "fp64":
            return st.lnps_pert()
        return torch.log1p(st.ps / self.ps_bar)

    def _ps(self, pi):
        """ps' = ps_bar (exp(pi') - 1) (state.py:81-83); expm1 in FP32."""
        if self.precision == "fp64":
            return self.ps_bar * (torch.exp(pi) - 1.0)
        return self.ps_bar * torch.expm1(pi)

    def implicit_ops(self, dt):
        """The operator list of ``implicit_step`` / ``implicit_step_adjoint``
        for a time step, in the working precision (IMPL_OPS order)."""
        integ, vg = self.m.integ, self.m.vg
        integ.semi.prepare(dt)
        integ.vdiff.prepare(dt)
        dmp = integ.dmp
        mv = integ.vdiff.minv
        opsl = [self.m.sp.laplace, dmp.kv, dmp.kd, dmp.ktt, dmp.kq, vg.ww, vg.tmtx, vg.gg,
                vg.dsig, integ.semi.minv] + [mv.get(n) for n in ("vor", "div", "t", "q")]
        if self.precision == "fp64":
            return opsl
        key = float(dt)
        if key not in self._iops:
            self._iops[key] = [None if x is None else x.to(self.rd).contiguous() for x in opsl]
        return self._iops[key]

    def _istep(self, dt, prev, tend):
        """Integrator.step in the working precision."""
        if self.precision == "fp64":
            return self.m.integ.step(dt, prev, tend)
        keys = ("vor", "div", "t", "pi", "q")
        c = lambda x: x.to(self.cd).contiguous()     # noqa: E731
        new = torch.ops.lbm_gb300.implicit_step(
            self.implicit_ops(dt), [c(prev[k]) for k in keys], [c(x) for x in tend],
            self.nmem, self.sp.nmax, self.vg.kmax, float(dt))
        return dict(zip(keys, new))

    def _ra(self, prev, cur, nxt):
        g = self.gamma
        return self._state(*(getattr(cur, k) + g * (getattr(prev, k) - 2.0 * getattr(cur, k)
                                                    + getattr(nxt, k)) for k in FIELDS))

    # ---- forward ------------------------------------------------------------
    def forward(self, ga, gb, dt, start, frc_t):
        """(ga, gb) -> (ga', gb') for one call of the reference loop: the
        operations of Dynamics.tendencies(ga), gb.to_spectral(),
        Integrator.step and load_spectral, with the transforms of one kind
        that share a call made in one launch over concatenated columns."""
        m, sp, K, nd = self.m, self.sp, self.vg.kmax, self.nd
        vo, di = sp.uv_to_vordiv(_cat([ga.u, gb.u], nd), _cat([ga.v, gb.v], nd))
        s = sp.grid_to_wave(_cat([self._pi(ga), gb.t, gb.q, self._pi(gb)], nd))
        g = sp.wave_to_grid(_cat([vo[..., :K], di[..., :K]], nd))
        pix, piy = sp.hgrad(s[..., 0])
        o = self.dyn._grid_kernel(ga, g[..., :K], g[..., K:], pix, piy, frc_t, None, None,
                                  want_omega=False)
        w = sp.grid_to_wave(_cat([o["gt_pi"], o["gt"], o["ke"], o["g"]], nd))
        fvo, fdi = sp.uv_to_vordiv(_cat([o["fu"], o["xu"], o["yu"]], nd),
                                   _cat([o["fv"], o["xv"], o["yv"]], nd))
        tend = (fvo[..., :K], fdi[..., :K] - sp.laplacian(w[..., K + 1:2 * K + 1]),
                -fdi[..., K:2 * K] + w[..., 1:K + 1], w[..., 0],
                -fdi[..., 2 * K:] + w[..., 2 * K + 1:])
        prev = {"vor": vo[..., K:], "div": di[..., K:], "t": s[..., 1:K + 1],
                "pi": s[..., 2 * K + 1], "q": s[..., K + 1:2 * K + 1]}
        new = self._istep(dt, prev, tend)
        u, v = sp.vordiv_to_uv(new["vor"], new["div"])
        gg = sp.wave_to_grid(_cat([new["t"], new["q"], new["pi"]], nd))
        gc = self._state(u, v, gg[..., :K], gg[..., K:2 * K],
                         self._ps(gg[..., 2 * K]))
        gb_new = ga if start else self._ra(gb, ga, gc)
        return gc, gb_new

    # ---- tangent-linear -----------------------------------------------------
    def _assemble(self, o):
        """The spectral tendencies from the grid kernel's outputs, in the
        operation order of Dynamics.tendencies (dynamics.py:186-262)."""
        sp = self.sp
        wt_pi = sp.grid_to_wave(o["gt_pi"])
        wt_t = sp.neg_divergence(o["xu"], o["xv"]) + sp.grid_to_wave(o["gt"])
        wt_vor, wt_div = sp.uv_to_vordiv(o["fu"], o["fv"])
        wt_div = wt_div - sp.laplacian(sp.grid_to_wave(o["ke"]))
        wt_q = sp.neg_divergence(o["yu"], o["yv"]) + sp.grid_to_wave(o["g"])
        return wt_vor, wt_div, wt_t, wt_pi, wt_q

    def tangent_tendencies(self, ga, dga, dfrc=None):
        """Tangent-linear of Dynamics.tendencies about the grid state ga."""
        sp = self.sp
        vor_s, div_s = sp.uv_to_vordiv(dga.u, dga.v)
        vor, div = sp.wave_to_grid(vor_s), sp.wave_to_grid(div_s)
        dpi = dga.ps / (self.ps_bar + ga.ps)
        pix, piy = sp.hgrad(sp.grid_to_wave(dpi))
        lin = None if self.linear else (ga.u, ga.v)
        o = self.dyn._grid_kernel(dga, vor, div, pix, piy, dfrc, None, None,
                                  want_omega=False, lin=lin)
        return self._assemble(o)

    def tangent(self, ga, gb, gc_ps, dga, dgb, dt, start, dfrc=None):
        """Tangent-linear step: (dga, dgb) -> (dga', dgb') about the trajectory
        (ga, gb) whose next level has surface pressure gc_ps."""
        sp = self.sp
        tend = self.tangent_tendencies(ga, dga, dfrc)
        vor, div = sp.uv_to_vordiv(dgb.u, dgb.v)
        prev = {"vor": vor, "div": div, "t": sp.grid_to_wave(dgb.t),
                "pi": sp.grid_to_wave(dgb.ps / (self.ps_bar + gb.ps)),
                "q": sp.grid_to_wave(dgb.q)}
        new = self._istep(dt, prev, tend)
        u, v = sp.vordiv_to_uv(new["vor"], new["div"])
        dgc = self._state(u, v, sp.wave_to_grid(new["t"]), sp.wave_to_grid(new["q"]),
                          (self.ps_bar + gc_ps) * sp.wave_to_grid(new["pi"]))
        dgb_new = dga if start else self._ra(dgb, dga, dgc)
        return dgc, dgb_new

    # ---- adjoint ------------------------------------------------------------
    def _tend_adjoint_kernel(self, ga, a_o):
        sp, vg, bs = self.sp, self.vg, self.bs
        J, I, K = sp.nlat, sp.nlon, vg.kmax
        named = {"dsig": vg.dsig, "sigm": vg.sigm, "alpha": vg.alpha, "w3": vg.w3, "wP": vg.wP,
                 "cpg": vg.cpg, "ww": vg.ww, "tmtx": vg.tmtx, "tref": vg.tbar, "ub": bs.u,
                 "vb": bs.v, "tb": bs.t, "qb": bs.q, "tvb": bs.tv, "absvor": bs.absvor,
                 "divb": bs.div, "x5b": bs.x5, "sdotb": bs.sdot, "pixb": bs.pix,
                 "piyb": bs.piy, "u0": None if self.linear else ga.u,
                 "v0": None if self.linear else ga.v}
        for k in ("fu", "fv", "ke", "gt", "xu", "xv", "g", "yu", "yv", "gt_pi"):
            named["a_" + k] = a_o[k].to(self.rd)
        outs = torch.ops.lbm_gb300.tendency_grid_adjoint(
            [named[k] for k in _ops.TADJ_INPUTS], self.nmem, J, I, K, [KAPPA, EPSVT, RAIR])
        return {k[2:]: t for k, t in zip(_ops.TADJ_OUTPUTS, outs)}

    def adjoint_tendencies(self, ga, aw):
        """Transpose of ``tangent_tendencies``: adjoints of the five spectral
        tendencies -> adjoint grid state (u v t q ps)."""
        tr, sp = self.tr, self.sp
        a_vor, a_div, a_t, a_pi, a_q = aw
        a_o = {"gt_pi": tr.grid_to_wave_T(a_pi), "gt": tr.grid_to_wave_T(a_t),
               "ke": tr.grid_to_wave_T(-sp.laplacian(a_div)), "g": tr.grid_to_wave_T(a_q)}
        a_o["xu"], a_o["xv"] = tr.neg_divergence_T(a_t)
        a_o["fu"], a_o["fv"] = tr.uv_to_vordiv_T(a_vor, a_div)
        a_o["yu"], a_o["yv"] = tr.neg_divergence_T(a_q)
        g = self._tend_adjoint_kernel(ga, a_o)
        a_pis = tr.hgrad_T(g["pix"], g["piy"])
        a_ps = tr.grid_to_wave_T(a_pis) / (self.ps_bar + ga.ps)
        du, dv = tr.uv_to_vordiv_T(tr.wave_to_grid_T(g["vor"]), tr.wave_to_grid_T(g["div"]))
        return _ns(u=g["u"] + du, v=g["v"] + dv, t=g["t"], q=g["q"], ps=a_ps)

    def _implicit_adjoint(self, dt, an):
        sp, vg = self.sp, self.vg
        keys = ("vor", "div", "t", "pi", "q")
        outs = torch.ops.lbm_gb300.implicit_step_adjoint(
            self.implicit_ops(dt), [an[k].to(self.cd) for k in keys], self.nmem, sp.nmax,
            vg.kmax, float(dt))
        return dict(zip(keys, outs[:5])), dict(zip(keys, outs[5:]))

    def adjoint(self, ga, gb, gc_ps, a_ga, a_gb, dt, start):
        """Transpose of ``tangent``: adjoints of (ga', gb') -> adjoints of
        (ga, gb), plus the adjoint of the spectral T tendency (whose
        grid-to-wave transpose is this step's heating gradient)."""
        tr, g = self.tr, self.gamma
        if start:
            a_c = a_ga
            a_a = a_gb
            a_b = None
        else:
            a_c = _ns(**{k: getattr(a_ga, k) + g * getattr(a_gb, k) for k in FIELDS})
            a_a = _ns(**{k: (1.0 - 2.0 * g) * getattr(a_gb, k) for k in FIELDS})
            a_b = _ns(**{k: g * getattr(a_gb, k) for k in FIELDS})
        K, sp, nd = self.vg.kmax, self.sp, self.nd
        # load_spectral
        an_vor, an_div = tr.vordiv_to_uv_T(a_c.u, a_c.v)
        x = tr.wave_to_grid_T(_cat([a_c.t, a_c.q, a_c.ps * (self.ps_bar + gc_ps)], nd))
        an = {"vor": an_vor, "div": an_div, "t": x[..., :K], "q": x[..., K:2 * K],
              "pi": x[..., 2 * K]}
        ap, aw = self._implicit_adjoint(dt, an)
        # grid-to-wave transposes of the tendencies of ga and of gb.to_spectral
        y = tr.grid_to_wave_T(_cat([aw["pi"], aw["t"], -sp.laplacian(aw["div"]), aw["q"],
                                    ap["t"], ap["q"], ap["pi"]], nd))
        z = torch.zeros_like(aw["t"])
        fu, fv = tr.uv_to_vordiv_T(_cat([aw["vor"], z, z], nd),
                                   _cat([aw["div"], -aw["t"], -aw["q"]], nd))
        a_o = {"gt_pi": y[..., 0], "gt": y[..., 1:K + 1], "ke": y[..., K + 1:2 * K + 1],
               "g": y[..., 2 * K + 1:3 * K + 1], "fu": fu[..., :K], "fv": fv[..., :K],
               "xu": fu[..., K:2 * K], "xv": fv[..., K:2 * K], "yu": fu[..., 2 * K:],
               "yv": fv[..., 2 * K:]}
        g = self._tend_adjoint_kernel(ga, a_o)
        a_ps = tr.grid_to_wave_T(tr.hgrad_T(g["pix"], g["piy"])) / (self.ps_bar + ga.ps)
        w2 = tr.wave_to_grid_T(_cat([g["vor"], g["div"]], nd))
        uu, vv = tr.uv_to_vordiv_T(_cat([ap["vor"], w2[..., :K]], nd),
                                   _cat([ap["div"], w2[..., K:]], nd))
        b = _ns(u=uu[..., :K], v=vv[..., :K], t=y[..., 3 * K + 1:4 * K + 1],
                q=y[..., 4 * K + 1:5 * K + 1], ps=y[..., 5 * K + 1] / (self.ps_bar + gb.ps))
        if a_b is not None:
            b = _ns(**{k: getattr(b, k) + getattr(a_b, k) for k in FIELDS})
        ta = _ns(u=g["u"] + uu[..., K:], v=g["v"] + vv[..., K:], t=g["t"], q=g["q"], ps=a_ps)
        a_prev = _ns(**{k: getattr(ta, k) + getattr(a_a, k) for k in FIELDS})
        return a_prev, b, aw["t"]


# ---------------------------------------------------------------------------
# Response and gradient
# ---------------------------------------------------------------------------
class AreaMeanStreamfunction:
    """Gaussian-weighted area mean of psi' = wave_to_grid(inv_laplacian(vor'))
    at the full level nearest ``sigma`` over a latitude/longitude box
    (bounds inclusive), from the final grid state's u, v."""

    def __init__(self, sp, vg, sigma=0.25, lat=(30.0, 60.0), lon=(150.0, 210.0)):
        self.sp = sp
        sig = np.asarray(vg.host("sig"))
        self.k = int(np.argmin(np.abs(sig - sigma)))
        box = response_box(np.asarray(sp.lat_deg), np.asarray(sp.lon_deg), lat[0], lat[1],
                           lon[0], lon[1])
        self.npts = (int(box.any(axis=1).sum()), int(box.any(axis=0).sum()))
        w = box * np.asarray(sp.gw)[:, None]
        w = w / w.sum()
        K = vg.kmax
        wk = np.zeros((sp.nlat, sp.nlon, K))
        wk[..., self.k] = w
        self.weights = torch.as_tensor(wk, device=sp.device)

    def __call__(self, st):
        sp = self.sp
        vor, _ = sp.uv_to_vordiv(st.u, st.v)
        psi = sp.wave_to_grid(sp.inverse_laplacian(vor))
        return (psi * self.weights).sum(dim=(-3, -2, -1))     # one value per member

    def seed(self, tr, like):
        """Adjoint grid state of the response (d J / d final state)."""
        sp = self.sp
        a_vor = sp.inverse_laplacian(tr.wave_to_grid_T(self.weights.expand_as(like.u)
                                                       .contiguous()))
        u, v = tr.uv_to_vordiv_T(a_vor, torch.zeros_like(a_vor))
        a = _zeros_like_state(like)
        a.u, a.v = u, v
        return a


class _GraphedCall:
    """A function of flat device tensors captured once as a CUDA graph:
    each call copies its arguments into the captured inputs and replays.
    The outputs are the graph's own buffers, overwritten by the next replay."""

    def __init__(self, fn, inputs, keep=()):
        self.keep = list(keep)            # tensors whose addresses the graph holds
        self.inputs = [x.clone() for x in inputs]
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            fn(*self.inputs)              # first use (lazy setup) outside the capture
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="relaxed"):
            self.outputs = fn(*self.inputs)

    def __call__(self, *inputs):
        torch._foreach_copy_(self.inputs, list(inputs))
        self.graph.replay()
        return self.outputs


def _flat(*states):
    return [getattr(st, k) for st in states for k in FIELDS]


class ForcingGradient:
    """J(heating) and dJ/d(heating) for a steady 3-D heating (K/s, the
    ``frc_t`` argument of every call), from the model's zero initial state,
    over the calls of ``LBM._schedule(nsteps)`` (start-up calls included).
    The reverse sweep re-advances from at most ``snaps`` stored states;
    ``snaps=None`` stores every call's state when they fit in ``mem_frac`` of
    the device memory free at construction (no re-steps: one forward sweep,
    then the adjoint calls), else as many as fit, up to ``MAX_SNAPS``, on the
    binomial schedule.  With ``use_graph`` every forward call and every adjoint call replays a
    CUDA graph of its (dt, start-up) variant; the kernels and their order
    are those of the eager calls, so the results are bitwise the same."""

    MAX_SNAPS = 256          # the binomial recursion's depth grows with the states

    def __init__(self, model, response, nsteps=None, ndays=None, snaps=None, use_graph=True,
                 pipeline=True, mem_frac=0.5, precision="fp64"):
        self.step = TimeStep(model, precision)
        self.use_graph = bool(use_graph)
        self.pipeline = bool(pipeline)
        self._fg, self._ag = {}, {}
        self.response = response
        if nsteps is None:
            nsteps = int(round((ndays if ndays is not None else model.cfg.ndays)
                               * model.cfg.steps_per_day))
        self.calls = model._schedule(nsteps)
        if snaps is None:
            snaps = self.auto_snaps(len(self.calls), self.state_bytes(), mem_frac)
        self.snaps = int(snaps)
        self.actions = binomial_schedule(len(self.calls), self.snaps)
        self.forward_steps = 0
        self.peak_stored = 0
        self._saved = None

    def state_bytes(self):
        """Device bytes of one stored (ga, gb) pair."""
        st = self.step
        cols = st.nmem * st.sp.nlat * st.sp.nlon
        return 2 * cols * (4 * st.vg.kmax + 1) * torch.empty(0, dtype=st.rd).element_size()

    @classmethod
    def auto_snaps(cls, ncalls, pair_bytes, mem_frac=0.5, free_bytes=None):
        """Stored states for ``ncalls`` calls: all of them (plus the one the
        last call makes) when they fit in ``mem_frac`` of ``free_bytes``
        (default: the device's free memory), else as many as fit, capped."""
        if free_bytes is None:
            free_bytes = torch.cuda.mem_get_info()[0]
        fit = int(mem_frac * free_bytes) // max(1, pair_bytes)
        if fit >= ncalls + 1:
            return ncalls
        return max(1, min(fit, cls.MAX_SNAPS))

    def _heating(self, heating):
        sp, vg = self.step.sp, self.step.vg
        h = to_device(heating, sp.device).to(self.step.rd)
        want = self.step._lead() + (sp.nlat, sp.nlon, vg.kmax)
        if tuple(h.shape) != want:
            raise ValueError(f"heating must be ([nmem,] nlat, nlon, kmax) = {want}, "
                             f"got {tuple(h.shape)}")
        return h.contiguous()

    def _fwd_call(self, cur, s, h):
        st = self.step
        dt, start = self.calls[s]
        if not self.use_graph:
            return st.forward(*cur, dt, start, h)
        g = self._fg.get((dt, start))
        flat = _flat(*cur) + [h]
        if g is None:
            def fn(*x):
                gc, gbn = st.forward(st._state(*x[0:5]), st._state(*x[5:10]), dt, start, x[10])
                out = _flat(gc, gbn)
                return [o.clone() if any(o is i for i in x) else o for o in out]
            g = self._fg[(dt, start)] = _GraphedCall(fn, flat, st.resources())
        out = g(*flat)
        return st._state(*out[0:5]), st._state(*out[5:10])

    def _adj_call(self, cur, next_ps, a_ga, a_gb, s):
        st = self.step
        dt, start = self.calls[s]
        if not self.use_graph:
            return st.adjoint(cur[0], cur[1], next_ps, a_ga, a_gb, dt, start)
        g = self._ag.get((dt, start))
        flat = _flat(*cur) + [next_ps] + _flat(a_ga, a_gb)
        if g is None:
            def fn(*x):
                a, b, w = st.adjoint(st._state(*x[0:5]), st._state(*x[5:10]), x[10],
                                     _ns(**dict(zip(FIELDS, x[11:16]))),
                                     _ns(**dict(zip(FIELDS, x[16:21]))), dt, start)
                return _flat(a, b) + [w]
            g = self._ag[(dt, start)] = _GraphedCall(fn, flat, st.resources())
        out = g(*flat)
        return (_ns(**dict(zip(FIELDS, out[0:5]))), _ns(**dict(zip(FIELDS, out[5:10]))),
                out[10])

    def _own(self, st):
        """A state that later graph replays cannot overwrite."""
        return self.step._state(*(x.clone() for x in _flat(st))) if self.use_graph else st

    def _advance(self, cur, i, j, h):
        for s in range(i, j):
            cur = self._fwd_call(cur, s, h)
            self.forward_steps += 1
        return cur

    def forward(self, heating):
        """Forward sweep; returns J (0-d device tensor) and keeps the stored
        states for ``backward``."""
        h = self._heating(heating)
        z = self.step.zero_state()
        cur, pos, slots = (z, z), 0, {}
        self.forward_steps, self.peak_stored = 0, 0
        n = len(self.calls)
        i = 0
        acts = self.actions
        while acts[i][0] != "adjoint":
            cur, pos = self._do(acts[i], cur, pos, slots, h)
            i += 1
        # the last call: state n (the response); its ps' is the next level of
        # call n - 1 in the reverse sweep
        last = self._own(self._advance(cur, n - 1, n, h)[0])
        J = self.response(last)
        self._saved = (h, i, cur, pos, slots, last.ps, last)
        return J

    def _do(self, act, cur, pos, slots, h):
        kind = act[0]
        if kind == "store":
            cur = (self._own(cur[0]), self._own(cur[1]))
            slots[act[1]] = cur
            self.peak_stored = max(self.peak_stored, len(slots))
        elif kind == "restore":
            cur, pos = slots[act[1]], act[1]
        elif kind == "advance":
            cur, pos = self._advance(cur, act[1], act[2], h), act[2]
        elif kind == "free":
            slots.pop(act[1])
        return cur, pos

    def backward(self):
        """Reverse sweep; returns dJ/d(heating) on the grid."""
        if self._saved is None:
            raise RuntimeError("backward() needs a forward() first")
        h, i, cur, pos, slots, next_ps, final = self._saved
        st = self.step
        a_ga = self.response.seed(st.tr, final)
        a_gb = _zeros_like_state(final)
        if self.use_graph and self.pipeline:
            g = self._backward_pipelined(h, i, cur, pos, slots, next_ps, a_ga, a_gb)
            self._saved = None
            return g
        acc = None
        for act in self.actions[i:]:
            if act[0] != "adjoint":
                cur, pos = self._do(act, cur, pos, slots, h)
                continue
            s = act[1]
            if pos != s:
                raise RuntimeError(f"checkpoint schedule out of step: at {pos}, reversing {s}")
            a_ga, a_gb, a_wt = self._adj_call(cur, next_ps, a_ga, a_gb, s)
            acc = a_wt.clone() if acc is None else acc + a_wt
            next_ps = cur[0].ps.clone() if self.use_graph else cur[0].ps
            pos = None
        self._saved = None
        return st.tr.grid_to_wave_T(acc)

    def _backward_pipelined(self, h, i, cur, pos, slots, next_ps, a_ga, a_gb, depth=3):
        """The reverse sweep on two streams.  The schedule's restore /
        advance / store actions depend only on stored states, never on
        adjoint results, so they run ahead on a second stream and hand each
        state to be reversed through a ring of ``depth`` buffers; the adjoint
        calls run on the current stream, each after an event for its state,
        and each buffer is refilled only after an event that its adjoint call
        has read it.  Both streams replay CUDA graphs; one member's kernels
        leave most of the GPU idle, so the two chains overlap."""
        st = self.step
        main = torch.cuda.current_stream()
        side = torch.cuda.Stream()
        # every graph variant exists before the two streams start
        for s in range(len(self.calls)):
            dt, start = self.calls[s]
            if (dt, start) not in self._ag:
                self._adj_call(cur, next_ps, a_ga, a_gb, s)
        # the ring is made on the main stream before the side stream is
        # ordered after it: the side stream's first copies into the ring must
        # not overtake these clones
        ring = [(self._own(cur[0]), self._own(cur[1])) for _ in range(depth)]
        side.wait_stream(main)
        # stored states made on the main stream are read (and dropped) by the
        # side stream: their memory must not be reused before it is done
        for pair in list(slots.values()) + [cur]:
            for x in _flat(*pair):
                x.record_stream(side)
        freed = [None] * depth
        acc, k = None, 0
        for act in self.actions[i:]:
            if act[0] != "adjoint":
                with torch.cuda.stream(side):
                    cur, pos = self._do(act, cur, pos, slots, h)
                continue
            s = act[1]
            if pos != s:
                raise RuntimeError(f"checkpoint schedule out of step: at {pos}, reversing {s}")
            slot = k % depth
            with torch.cuda.stream(side):
                if freed[slot] is not None:
                    side.wait_event(freed[slot])
                torch._foreach_copy_(_flat(*ring[slot]), _flat(*cur))
                ready = torch.cuda.Event()
                ready.record(side)
            main.wait_event(ready)
            a_ga, a_gb, a_wt = self._adj_call(ring[slot], next_ps, a_ga, a_gb, s)
            acc = a_wt.clone() if acc is None else acc + a_wt
            next_ps = ring[slot][0].ps.clone()
            freed[slot] = torch.cuda.Event()
            freed[slot].record(main)
            pos, k = None, k + 1
        main.wait_stream(side)
        return st.tr.grid_to_wave_T(acc)

    def value_and_grad(self, heating):
        J = self.forward(heating)
        return J, self.backward()

    def tangent(self, heating, direction):
        """Tangent-linear response dJ(heating; direction), the forward and the
        tangent-linear model run side by side (the response is linear)."""
        h, d = self._heating(heating), self._heating(direction)
        st = self.step
        z = st.zero_state()
        cur, dcur = (z, z), (z, z)
        for dt, start in self.calls:
            nxt = st.forward(*cur, dt, start, h)      # eager: the trajectory is kept
            dcur = st.tangent(cur[0], cur[1], nxt[0].ps, *dcur, dt, start, dfrc=d)
            cur = nxt
        return self.response(dcur[0])

    def value(self, heating):
        """J alone, by a plain forward run (no stored states)."""
        h = self._heating(heating)
        z = self.step.zero_state()
        cur = (z, z)
        for s in range(len(self.calls)):
            cur = self._fwd_call(cur, s, h)
        return self.response(cur[0])


class HeatingResponse(torch.autograd.Function):
    """``J = HeatingResponse.apply(heating, gradient)`` with a
    ``ForcingGradient``; ``J.backward()``
    runs the checkpointed adjoint and fills ``heating.grad``."""

    @staticmethod
    def forward(ctx, heating, gradient):
        ctx.gradient = gradient
        with torch.no_grad():
            return gradient.forward(heating.detach())

    @staticmethod
    def backward(ctx, gJ):
        g = ctx.gradient.backward()
        gJ = gJ.reshape(gJ.shape + (1,) * (g.dim() - gJ.dim()))   # one J per member
        return gJ * g, None
