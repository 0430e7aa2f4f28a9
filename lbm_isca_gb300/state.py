"""Perturbation state in grid space (drop-in for pylbm_isca/state.py:26-148).

The fields are device tensors.  The ensemble stepper keeps its own packed
spectral copy while it integrates and writes the grid fields back here when
a run ends; this class is the user-facing view, with the reference's exact
pi' = ln(ps_bar + ps') - ln(ps_bar) round trip.
"""

from __future__ import annotations

import numpy as np
import torch

from .backend import asnumpy, resolve, to_device


class State:
    """Perturbation fields u, v, t, q ((E,) J, I, K) and ps ((E,) J, I) [hPa]."""

    __slots__ = ("xp", "device", "u", "v", "t", "q", "ps", "ps_bar", "lnps_bar")

    def __init__(self, ps_bar, u=None, v=None, t=None, q=None, ps=None, device="auto",
                 xp=None):
        self.xp = torch
        if isinstance(device, torch.device):
            self.device = device
        else:
            self.device = resolve(device)
        dev = self.device
        self.ps_bar = to_device(ps_bar, dev)
        self.lnps_bar = torch.log(self.ps_bar)
        shape3 = None
        for f in (u, v, t, q):
            if f is not None:
                shape3 = tuple(f.shape)
                break
        if shape3 is None:
            raise ValueError("need at least one 3-D field to infer the shape")
        z3 = lambda: torch.zeros(shape3, device=dev, dtype=torch.float64)  # noqa: E731
        self.u = z3() if u is None else to_device(u, dev)
        self.v = z3() if v is None else to_device(v, dev)
        self.t = z3() if t is None else to_device(t, dev)
        self.q = z3() if q is None else to_device(q, dev)
        self.ps = (torch.zeros(tuple(self.ps_bar.shape), device=dev, dtype=torch.float64)
                   if ps is None else to_device(ps, dev))

    @classmethod
    def zeros(cls, ps_bar, nlev, device="auto", xp=None):
        nlat, nlon = tuple(ps_bar.shape)
        dev = device if isinstance(device, torch.device) else resolve(device)
        return cls(ps_bar, u=torch.zeros((nlat, nlon, nlev), device=dev, dtype=torch.float64),
                   device=dev)

    @classmethod
    def zeros_ensemble(cls, ps_bar, nlev, nmem, device="auto", xp=None):
        """Member axis first: (nmem, nlat, nlon, nlev) / (nmem, nlat, nlon)."""
        nlat, nlon = tuple(ps_bar.shape)
        dev = device if isinstance(device, torch.device) else resolve(device)
        obj = cls(ps_bar, u=torch.zeros((nmem, nlat, nlon, nlev), device=dev,
                                        dtype=torch.float64), device=dev)
        obj.ps = torch.zeros((nmem, nlat, nlon), device=dev, dtype=torch.float64)
        return obj

    def copy(self):
        return State(self.ps_bar, self.u.clone(), self.v.clone(), self.t.clone(),
                     self.q.clone(), self.ps.clone(), device=self.device)

    def lnps_pert(self):
        """pi' = ln(ps_bar + ps') - ln(ps_bar)  (state.py:77-79)."""
        return torch.log(self.ps_bar + self.ps) - self.lnps_bar

    def set_from_lnps(self, pi):
        """ps' = ps_bar (exp(pi') - 1)  (state.py:81-83)."""
        pi = to_device(pi, self.device)
        self.ps = self.ps_bar * (torch.exp(pi) - 1.0)

    def to_spectral(self, sp):
        vor, div = sp.uv_to_vordiv(self.u, self.v)
        return {"vor": vor, "div": div, "t": sp.grid_to_wave(self.t),
                "pi": sp.grid_to_wave(self.lnps_pert()), "q": sp.grid_to_wave(self.q)}

    def load_spectral(self, sp, spec):
        self.u, self.v = sp.vordiv_to_uv(spec["vor"], spec["div"])
        self.t = sp.wave_to_grid(spec["t"])
        self.q = sp.wave_to_grid(spec["q"])
        self.set_from_lnps(sp.wave_to_grid(spec["pi"]))
        return self

    def assign(self, other):
        self.u = other.u.clone()
        self.v = other.v.clone()
        self.t = other.t.clone()
        self.q = other.q.clone()
        self.ps = other.ps.clone()
        return self

    def robert_asselin(self, current, new, gamma=0.04):
        """X_f(t) = X(t) + gamma [X(t-dt) - 2 X(t) + X(t+dt)] (state.py:110-128)."""
        for name in ("u", "v", "t", "q", "ps"):
            prev = getattr(self, name)
            cur = getattr(current, name)
            nxt = getattr(new, name)
            setattr(self, name, cur + gamma * (prev - 2.0 * cur + nxt))
        return self

    def max_abs(self):
        return {k: float(getattr(self, k).abs().max()) for k in ("u", "v", "t", "ps", "q")}

    def isfinite(self):
        return all(bool(torch.isfinite(getattr(self, k)).all())
                   for k in ("u", "v", "t", "q", "ps"))

    def to_numpy(self):
        return {k: asnumpy(getattr(self, k)) for k in ("u", "v", "t", "q", "ps")}
