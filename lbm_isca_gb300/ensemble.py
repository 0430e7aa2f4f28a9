"""Ensemble batching (drop-in for pylbm_isca/ensemble.py:41-165).

The reference folds the member axis into the transform columns and unfolds
after every transform (ensemble.py:55-72).  Here the member axis is the
batch dimension of every lbm_gb300 kernel, so nothing is folded: the
transforms read the (E, ...) arrays in place, and the fused stepper keeps
members as the outermost axis of its packed spectral state.
"""

from __future__ import annotations

import numpy as np
import torch

from .backend import resolve, to_device
from .model import LBM, Config
from .spectral import Spectral
from .vertical import VerticalGrid


class BatchedSpectral(Spectral):
    """A Spectral whose arrays carry a leading member axis (ensemble.py:41-106)."""

    batched = True


class EnsembleForcing:
    """Constant per-member temperature forcing with the MJO-forcing protocol
    (ensemble.py:109-121): ``step()`` returns the same (E, nlat, nlon, K)
    array on every call."""

    def __init__(self, gtf, xp=None, device="auto"):
        self.gtf = to_device(gtf, resolve(device))

    def step(self):
        return self.gtf


def build_heating_sweep(base_heat, nmem, mode="longitude", xp=np):
    """Heating fields from one base field (ensemble.py:124-149)."""
    base = np.asarray(base_heat.detach().cpu() if isinstance(base_heat, torch.Tensor)
                      else base_heat)
    nlat, nlon, kmax = base.shape
    out = np.empty((nmem, nlat, nlon, kmax), dtype=np.float64)
    if mode == "longitude":
        for e in range(nmem):
            out[e] = np.roll(base, int(round(e * nlon / nmem)), axis=1)
    elif mode == "amplitude":
        for e, s in enumerate(np.linspace(0.5, 1.5, nmem)):
            out[e] = s * base
    else:
        raise ValueError(mode)
    return out


def make_ensemble_model(basic_state, nmem, config=None, device="gpu", nlon=None,
                        nlat=None, nmax=None, sigm=None):
    """(model, batched_spectral, vertical_grid) for `nmem` members on one GPU
    (ensemble.py:152-165).  The grid defaults to the reference's T42L20; the
    extra keywords select another truncation or level set."""
    kw = {}
    if nlon is not None:
        kw = dict(nlon=nlon, nlat=nlat, nmax=nmax)
    sp_plain = Spectral(device=device, **kw)
    sp_batch = BatchedSpectral(device=device, **kw)
    vg = VerticalGrid(device=device) if sigm is None else VerticalGrid(sigm=sigm,
                                                                        device=device)
    cfg = config or Config()
    cfg.nmem = nmem
    model = LBM(basic_state, sp_batch, vg, cfg, basic_spectral=sp_plain)
    return model, sp_batch, vg
