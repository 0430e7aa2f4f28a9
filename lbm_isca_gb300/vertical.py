"""Simmons-Burridge sigma coordinate (drop-in for pylbm_isca/vertical.py:50-216).

The operators are K-vectors and K x K matrices built once from the half
levels (vertical.py:59-129) and from the reference virtual-temperature
profile (vertical.py:139-193).  They are assembled in FP64 on the host, where
they cost microseconds, and moved to the device once; the time step consumes
them fused into the lbm_gb300 kernels (the hydrostatic matrix and the
energy-conversion operator are applied column by column inside the
grid-point tendency kernel and the implicit-update kernel).
"""

from __future__ import annotations

import numpy as np
import torch

from .backend import asnumpy, resolve
from .constants import KAPPA, RAIR, SIGM


class VerticalGrid:
    """Sigma half levels and their Simmons-Burridge operators."""

    _DEVICE_ATTRS = ("dsig", "sig", "sigm", "dsigm", "alpha", "dlog3", "cpg", "w3", "wP",
                     "ww")
    _DEVICE_ATTRS_TBAR = ("tbar", "gg", "tmtx", "whmtx", "gcmtx")

    def __init__(self, sigm=SIGM, kappa=KAPPA, device="auto"):
        self.device = resolve(device)
        self.xp = torch
        sigm = np.asarray(asnumpy(sigm), dtype=np.float64)
        self.kmax = K = sigm.size - 1
        self.kappa = kappa
        h = {"sigm": sigm}
        bot, top = sigm[:-1], sigm[1:]
        h["dsig"] = bot - top
        safe = np.where(top > 0.0, top, 1.0)
        lr = np.log(bot) - np.log(safe)
        # alpha with the massless-top limit alpha = 1 (vertical.py:343-347)
        h["alpha"] = 1.0 - np.where(top > 0.0, top * lr / (bot - top), 0.0)
        h["sig"] = bot * np.exp(-h["alpha"])
        h["dlog1"] = h["alpha"].copy()
        h["dlog2"] = np.where(top > 0.0, np.log(h["sig"]) - np.log(safe), 0.0)
        h["dlog3"] = np.where(top > 0.0, lr, 0.0)
        h["cpg"] = (bot * h["dlog1"] + top * h["dlog2"]) / h["dsig"]
        h["w3"] = h["dlog3"] / h["dsig"]
        h["wP"] = h["alpha"] - h["cpg"]
        dsm = np.empty(K + 1)
        dsm[0] = sigm[0] - h["sig"][0]
        dsm[1:K] = h["sig"][:-1] - h["sig"][1:]
        dsm[K] = h["sig"][-1] - sigm[-1]
        h["dsigm"] = dsm
        ww = np.tril(np.ones((K, K)), -1) * (RAIR * h["dlog3"])[None, :]
        ww[np.arange(K), np.arange(K)] = RAIR * h["alpha"]
        h["ww"] = ww
        self._h = h
        for name, val in h.items():
            if name in self._DEVICE_ATTRS:
                setattr(self, name, torch.as_tensor(val, device=self.device))
            else:
                setattr(self, name, val)
        self.tbar = self.gg = self.tmtx = self.whmtx = self.gcmtx = None

    def host(self, name):
        """FP64 host copy of an operator (numpy)."""
        return self._h[name]

    def set_reference_temperature(self, tbar):
        """Reference-Tv operators gg, tmtx, whmtx, gcmtx (vertical.py:410-464)."""
        K = self.kmax
        tb = np.array(asnumpy(tbar), dtype=np.float64).reshape(K)
        h = self._h
        h["tbar"] = tb
        h["gg"] = RAIR * tb * h["cpg"]
        above = np.triu(np.ones((K, K)), 1) * h["dsig"][None, :]
        tm = KAPPA * tb[:, None] * h["w3"][:, None] * above
        tm[np.arange(K), np.arange(K)] = KAPPA * tb * h["alpha"]
        h["tmtx"] = tm
        h["whmtx"] = h["ww"] @ tm
        h["gcmtx"] = np.outer(h["gg"], h["dsig"])
        for name in self._DEVICE_ATTRS_TBAR:
            setattr(self, name, torch.as_tensor(h[name], device=self.device))

    def hydrostatic(self, tv):
        """phi = Tv @ WW.T over the last (level) axis (vertical.py:467-474)."""
        t = tv if isinstance(tv, torch.Tensor) else torch.as_tensor(np.asarray(tv))
        t = t.to(self.device)
        return t @ self.ww.to(t.dtype).T


def compute_tbar(gft):
    """Plain mean over the (nlat, nlon) grid (vertical.py:477-487)."""
    if isinstance(gft, torch.Tensor):
        return gft.sum(dim=(0, 1)) / (gft.shape[0] * gft.shape[1])
    g = np.asarray(gft)
    return g.sum(axis=(0, 1)) / (g.shape[0] * g.shape[1])
