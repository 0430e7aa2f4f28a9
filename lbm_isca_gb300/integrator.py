"""Semi-implicit leapfrog integration (drop-in for pylbm_isca/integrator.py).

Damping coefficients are (n, k) arrays built once on the host (they are a
few hundred numbers).  The per-n gravity-wave matrices are assembled and
inverted in FP64 on the device (``lbm_gravity_wave_matrices`` and
``lbm_batched_inverse``, replacing integrator.py:149-161); so are the
implicit vertical-diffusion operators (integrator.py:216-228).  The
condition numbers the reference records (integrator.py:163) are computed
on the host from the device matrices.  ``Integrator.step`` is one launch of
``lbm_implicit_step``.
"""

from __future__ import annotations

import numpy as np
import torch

from . import ops as _ops
from .backend import asnumpy
from .constants import S2D


def _to_seconds(value, unit):
    u = unit.strip().upper()[:3]
    return float(value) * {"SEC": 1.0, "MIN": 60.0, "HOU": 3600.0, "DAY": 86400.0,
                           "MON": 30 * 86400.0}[u]


def _drag(d, kmax, tunit):
    """Per-level damping timescales -> s^-1, <= 0 disables (integrator.py:101-112)."""
    out = np.zeros(kmax)
    if d is None:
        return out
    d = np.asarray(d, dtype=np.float64)
    if d.size != kmax:
        raise ValueError(f"damping profile must have {kmax} entries")
    sec = np.array([_to_seconds(x, tunit) for x in d])
    good = sec > 0
    out[good] = 1.0 / sec[good]
    return out


class Damping:
    """Hyperdiffusion, sponge and Rayleigh/Newtonian drag (integrator.py:33-98)."""

    def __init__(self, sp, vgrid, order=4, tefold=2.0, tunit_hdif="HOUR", ddragv=None,
                 ddragd=None, ddragt=None, ddragq=None, tunit_damp="DAY", ray0=30.0,
                 zsclh=8.0e3, rzsclh=7.0e3, sponge=True):
        self.sp, self.vg = sp, vgrid
        nmax, kmax = sp.nmax, vgrid.kmax
        n = np.arange(nmax + 1, dtype=np.float64)
        nn1 = n * (n + 1.0)
        p = order // 2
        tau = _to_seconds(tefold, tunit_hdif)
        difmax = (nmax * (nmax + 1.0) / nmax) ** p
        dift_n = (nn1 / nmax) ** p
        difv_n = dift_n - (2.0 / nmax) ** p
        kt = (1.0 / tau) * dift_n / difmax
        kv = (1.0 / tau) * difv_n / difmax
        kt[0] = 0.0
        kv[0] = 0.0
        kv[1] = max(kv[1], 0.0)
        self.kt_h, self.kv_h = kt, kv
        self.sponge_k = np.zeros(kmax)
        if sponge:
            ray0_s = _to_seconds(ray0, tunit_hdif)
            sig = vgrid.host("sig")
            z = -zsclh * np.log(sig)
            rzofs = -zsclh * np.log(float(sig[-1]))
            self.sponge_k = np.maximum(1.0 + np.tanh((z - rzofs) / rzsclh), 1e-20) / ray0_s
        self.drag_v = _drag(ddragv, kmax, tunit_damp)
        self.drag_d = _drag(ddragd, kmax, tunit_damp)
        self.drag_t = _drag(ddragt, kmax, tunit_damp)
        self.drag_q = _drag(ddragq, kmax, tunit_damp)
        self.h = {"kv": kv[:, None] + self.sponge_k[None, :] + self.drag_v[None, :],
                  "kd": kv[:, None] + self.sponge_k[None, :] + self.drag_d[None, :],
                  "ktt": kt[:, None] + self.drag_t[None, :],
                  "kq": kt[:, None] + self.drag_q[None, :]}
        dev = sp.device
        for k, val in self.h.items():
            setattr(self, k, torch.as_tensor(val, device=dev))


def batched_inverse(a):
    """FP64 batched inverse on the device (Gauss-Jordan, partial pivoting)."""
    out, info = torch.ops.lbm_gb300.batched_inverse(a.contiguous().to(torch.float64))
    if int(info.max()) != 0:
        raise np.linalg.LinAlgError("singular matrix in batched inverse")
    return out


class SemiImplicit:
    """Gravity-wave matrices M(n) and their inverses (integrator.py:121-172)."""

    def __init__(self, sp, vgrid, damping):
        self.sp, self.vg, self.dmp = sp, vgrid, damping
        self._dt = None
        self.minv = None
        self._cache = {}

    def matrices(self, dt):
        """(M, Minv, cond) for a time step, computed once per distinct dt."""
        dt = float(dt)
        if dt not in self._cache:
            sp, vg, dmp = self.sp, self.vg, self.dmp
            mats = torch.ops.lbm_gb300.gravity_wave_matrices(
                sp.laplace, dmp.ktt, dmp.kd, vg.whmtx, vg.gcmtx, dt)
            minv = batched_inverse(mats)
            cond = np.array([np.linalg.cond(x) for x in asnumpy(mats)])
            self._cache[dt] = (mats, minv, cond)
        return self._cache[dt]

    def prepare(self, dt):
        if self._dt == dt:
            return
        self.m, self.minv, self.cond = self.matrices(dt)
        self._dt = dt

    def solve(self, rhs):
        """Apply M(n)^-1 over the (..., m, n, k) spectral layout."""
        mi = self.minv.to(rhs.dtype if torch.is_complex(rhs) else torch.float64)
        return torch.einsum("nij,...nj->...ni", mi, rhs)


class VerticalDiffusion:
    """Implicit sigma-space vertical diffusion (integrator.py:175-253)."""

    def __init__(self, vgrid, vdifv=None, vdifd=None, vdift=None, vdifq=None):
        self.vg = vgrid
        K = vgrid.kmax
        dsig, dsigm = vgrid.host("dsig"), vgrid.host("dsigm")
        a = np.zeros(K)
        c = np.zeros(K)
        a[1:] = 1.0 / (dsig[1:] * dsigm[1:K])
        c[:-1] = 1.0 / (dsig[:-1] * dsigm[1:K])
        b = -(a + c)
        c[0] = (dsigm[0] + dsigm[1]) / (dsig[0] * dsigm[0] * dsigm[1])
        a[0] = 0.0
        b[0] = -c[0]
        a[-1] = (dsigm[K - 1] + dsigm[K]) / (dsig[-1] * dsigm[K - 1] * dsigm[K])
        c[-1] = 0.0
        b[-1] = -a[-1]
        self.lop = np.diag(b) + np.diag(a[1:], -1) + np.diag(c[:-1], 1)
        self.coef = {name: _vdif_coef(v, K) for name, v in
                     (("vor", vdifv), ("div", vdifd), ("t", vdift), ("q", vdifq))}
        self._dt = None
        self.minv = {}
        self._cache = {}

    def operators(self, dt):
        dt = float(dt)
        if dt not in self._cache:
            K = self.vg.kmax
            dev = self.vg.device
            out = {}
            for name, nu in self.coef.items():
                if nu is None:
                    out[name] = None
                else:
                    a = torch.as_tensor(np.eye(K) - dt * nu[:, None] * self.lop,
                                        device=dev)[None]
                    out[name] = batched_inverse(a)[0]
            self._cache[dt] = out
        return self._cache[dt]

    def prepare(self, dt):
        if self._dt == dt:
            return
        self.minv = self.operators(dt)
        self._dt = dt

    def apply(self, field, name, skip_low_n=False):
        minv = self.minv.get(name)
        if minv is None:
            return field
        out = torch.einsum("ij,...j->...i", minv.to(field.dtype), field)
        if skip_low_n:
            out[..., 0, :] = field[..., 0, :]
            out[..., 1, :] = field[..., 1, :]
        return out


def _vdif_coef(v, kmax):
    if v is None:
        return None
    v = np.atleast_1d(np.asarray(v, dtype=np.float64))
    if v.size == 1:
        v = np.full(kmax, v[0])
    if np.any(v <= 0):
        return None
    return 1.0 / (S2D * v)


class Integrator:
    """Semi-implicit leapfrog step (integrator.py:256-315) as one kernel launch."""

    def __init__(self, sp, vgrid, damping, semi, vdiff):
        self.sp, self.vg = sp, vgrid
        self.dmp, self.semi, self.vdiff = damping, semi, vdiff

    def step(self, dt, prev, tend):
        sp, vg, dmp = self.sp, self.vg, self.dmp
        self.semi.prepare(dt)
        self.vdiff.prepare(dt)
        keys = ("vor", "div", "t", "pi", "q")

        def dev(x):
            t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x))
            return t.to(device=sp.device, dtype=torch.complex128).contiguous()
        pv = {k: dev(prev[k]) for k in keys}
        tv = dict(zip(keys, (dev(x) for x in tend)))
        K = vg.kmax
        batched = pv["vor"].dim() == 4
        E = pv["vor"].shape[0] if batched else 1
        mv = self.vdiff.minv
        opsl = [sp.laplace, dmp.kv, dmp.kd, dmp.ktt, dmp.kq, vg.ww, vg.tmtx, vg.gg, vg.dsig,
                self.semi.minv] + [mv.get(n) for n in ("vor", "div", "t", "q")]
        new = torch.ops.lbm_gb300.implicit_step(opsl, [pv[k] for k in keys],
                                                [tv[k] for k in keys], E, sp.nmax, K,
                                                float(dt))
        return dict(zip(keys, new))
