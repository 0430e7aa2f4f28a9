"""Spectral regridding between Gaussian grids / truncations (drop-in for
pylbm_isca/regrid.py).

A field moves native grid -> spectral (native truncation) -> zero-padded or
truncated coefficients -> target grid (regrid.py:1-31): the coefficient
normalisation does not depend on the grid or the truncation, so resizing is
padding or dropping the high-n tail.  Winds go through vorticity and
divergence.  Both transforms run in the lbm_gb300 kernels; results come back
as host arrays, as the reference's do.
"""

from __future__ import annotations

import numpy as np
import torch

from .backend import asnumpy


def detect_grid(path):
    """(nlon, nlat) of a Fortran-sequential field file, from its first record
    marker, assuming nlon = 2 nlat (regrid.py:45-64)."""
    with open(path, "rb") as fh:
        nbytes = int(np.frombuffer(fh.read(4), dtype=">i4")[0])
    if nbytes <= 0 or nbytes % 4:
        raise ValueError(f"{path}: unreadable record marker {nbytes}")
    npts = nbytes // 4
    nlat = int(round((npts / 2.0) ** 0.5))
    nlon = 2 * nlat
    if nlon * nlat != npts:
        raise ValueError(f"{path}: {npts} points per record is not a 2:1 Gaussian grid; "
                         f"pass the source grid explicitly")
    return nlon, nlat


def _same(a, b):
    return (a.nlon, a.nlat, a.nmax) == (b.nlon, b.nlat, b.nmax)


def _resize_spec(xi, dst_nmax):
    """Zero-pad or truncate spectral coefficients [m, n, ...] to dst_nmax."""
    m_src = xi.shape[0]
    m_dst = dst_nmax + 1
    if m_src == m_dst:
        return xi
    k = min(m_src, m_dst)
    out = torch.zeros((m_dst, m_dst) + tuple(xi.shape[2:]), dtype=xi.dtype, device=xi.device)
    out[:k, :k] = xi[:k, :k]
    return out


def regrid_scalar(src_sp, dst_sp, field):
    """A scalar grid field (2-D or 3-D) on ``dst_sp``'s grid (regrid.py:82-95)."""
    if _same(src_sp, dst_sp):
        return np.asarray(asnumpy(field))
    xi = _resize_spec(src_sp.grid_to_wave(field), dst_sp.nmax)
    return asnumpy(dst_sp.wave_to_grid(xi))


def regrid_uv(src_sp, dst_sp, u, v):
    """A horizontal wind through vorticity and divergence (regrid.py:98-108)."""
    if _same(src_sp, dst_sp):
        return np.asarray(asnumpy(u)), np.asarray(asnumpy(v))
    vor, div = src_sp.uv_to_vordiv(u, v)
    u2, v2 = dst_sp.vordiv_to_uv(_resize_spec(vor, dst_sp.nmax),
                                 _resize_spec(div, dst_sp.nmax))
    return asnumpy(u2), asnumpy(v2)


def regrid_basic_state(bs, src_sp, dst_sp):
    """A basic state on ``dst_sp``'s grid (regrid.py:111-123)."""
    from .basicstate import BasicState
    u, v = regrid_uv(src_sp, dst_sp, bs.u, bs.v)
    return BasicState(u=u, v=v,
                      t=regrid_scalar(src_sp, dst_sp, bs.t),
                      q=regrid_scalar(src_sp, dst_sp, bs.q),
                      ps=regrid_scalar(src_sp, dst_sp, bs.ps),
                      lat_deg=np.asarray(dst_sp.lat_deg), lon_deg=np.asarray(dst_sp.lon_deg),
                      sig=getattr(bs, "sig", None),
                      source=getattr(bs, "source", "") + " (regridded)")


def regrid_mjo_forcing(mjo, src_sp, dst_sp):
    """Regrid an MJO heating record set (gtf[day][lat][lon][lev]) in place,
    all days and levels in one batched transform; the object is reset
    (regrid.py:126-138)."""
    if _same(src_sp, dst_sp):
        return mjo
    nday, nlat, nlon, nlev = mjo.gtf.shape
    stack = np.transpose(mjo.gtf, (1, 2, 0, 3)).reshape(nlat, nlon, nday * nlev)
    out = regrid_scalar(src_sp, dst_sp, stack)
    mjo.gtf = np.transpose(out.reshape(dst_sp.nlat, dst_sp.nlon, nday, nlev), (2, 0, 1, 3))
    mjo.reset()
    return mjo


def regrid_steady_forcing(steady, src_sp, dst_sp):
    """Regrid a steady forcing's vor, div, t and ps fields in place; all four
    are grid scalars (regrid.py:141-151)."""
    if _same(src_sp, dst_sp):
        return steady
    steady.vor = regrid_scalar(src_sp, dst_sp, steady.vor)
    steady.div = regrid_scalar(src_sp, dst_sp, steady.div)
    steady.t = regrid_scalar(src_sp, dst_sp, steady.t)
    steady.ps = regrid_scalar(src_sp, dst_sp, steady.ps)
    return steady
