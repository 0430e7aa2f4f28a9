"""Basic-state preprocessing (drop-in for pylbm_isca/basicstate.py).

ERA5 monthly pressure-level fields -> the model's sigma levels: read and
average months (host: a file format), surface pressure from geopotential
height, spectral smoothing, zonal-mean / eddy filter, pressure -> sigma by a
natural cubic spline in ln p.  The column work runs in the lbm_gb300 kernels
(``lbm_z2ps``, ``lbm_spline``, ``lbm_zonal_filter``; FP64), the smoothing in
the spectral transforms; the pipeline keeps its fields on the device and
returns host arrays, as the reference does.  Every public function takes
host or device arrays.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from ._lib import check, lib
from .backend import asnumpy, stream_handle
from .constants import IMAX, JMAX, PLEV17

UNDEF_IN = -9.999e20      # undefined value of the input files
XMISS = -999.0            # missing-value marker of the pipeline

# variables of a month in the pressure-level file, in order; relative
# humidity and omega are skipped
BS_VARS = ["z", "rhum", "q", "t", "u", "v", "omega"]
BS_KEEP = ["z", "q", "t", "u", "v"]


def _dev(a, device=None):
    dev = torch.device(device) if device is not None else torch.device("cuda")
    t = a if isinstance(a, torch.Tensor) else \
        torch.from_numpy(np.array(a, dtype=np.float64, copy=True))
    if dev.type != "cuda":
        raise RuntimeError("basic-state kernels need a CUDA device (there is no CPU path)")
    return t.to(device=dev, dtype=torch.float64).contiguous()


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _st():
    return C.c_void_p(stream_handle())


# ---------------------------------------------------------------------------
# Reading (basicstate.py:53-109)
# ---------------------------------------------------------------------------
def read_pressure_levels(path, kmo=1, navg=3, nlon=IMAX, nlat=JMAX, nlev=17,
                         nvar=7, nmonth=None, yflip=True):
    """Average ``navg`` months from month ``kmo`` (wrapping past the last one)
    of a pressure-level file: Fortran sequential records, big-endian real*4,
    one (nlon, nlat) field per record, ordered month -> variable -> level,
    rows south first (``yflip`` turns them north first).  A point equal to
    ``UNDEF_IN`` in any averaged month becomes ``XMISS``; the comparison is
    made on the values widened to double precision, as the reference makes
    it.  Returns (nlat, nlon, nlev) arrays of z, q, t, u, v."""
    npts = nlon * nlat
    words = np.fromfile(path, dtype=">f4")
    if words.size % (npts + 2):
        raise ValueError(f"{path}: not a whole number of Fortran records")
    recs = words.reshape(-1, npts + 2)
    count = recs[:, 0].view(">i4")
    if not np.all(count == npts * 4):
        raise ValueError(f"{path}: bad record markers - wrong endianness "
                         f"or grid size? (got {count[0]}, want {npts * 4})")
    fields = recs[:, 1:-1].reshape(-1, nlat, nlon).astype(np.float64)
    per_month = nvar * nlev
    if fields.shape[0] % per_month:
        raise ValueError(f"{path}: {fields.shape[0]} records is not a multiple of "
                         f"{per_month} (= {nvar} vars x {nlev} levels)")
    months = fields.shape[0] // per_month
    acc = {v: np.zeros((nlat, nlon, nlev)) for v in BS_KEEP}
    bad = {v: np.zeros((nlat, nlon, nlev), dtype=bool) for v in BS_KEEP}
    mo = kmo
    for _ in range(navg):
        first = (mo - 1) * per_month
        if first + per_month > fields.shape[0]:
            raise ValueError(f"{path}: month {mo} beyond end of file")
        for iv, name in enumerate(BS_VARS):
            if name not in BS_KEEP:
                continue
            blk = np.moveaxis(fields[first + iv * nlev:first + (iv + 1) * nlev], 0, -1)
            if yflip:
                blk = blk[::-1]
            bad[name] |= blk == UNDEF_IN
            acc[name] += blk / float(navg)
        mo = mo + 1 if mo < months else 1
    for name in BS_KEEP:
        acc[name][bad[name]] = XMISS
    return acc


# ---------------------------------------------------------------------------
# Column kernels
# ---------------------------------------------------------------------------
def _z2ps_dev(z, zs, plev):
    z = _dev(z)
    nk = z.shape[-1]
    ncol = z.numel() // nk
    zsd = _dev(np.broadcast_to(asnumpy(zs), z.shape[:-1])) if zs is not None else None
    pl = _dev(plev)
    ps = torch.empty(z.shape[:-1], dtype=torch.float64, device=z.device)
    check(lib().lbm_z2ps(ncol, nk, _p(z), _p(zsd), _p(pl), _p(ps), _st()), "lbm_z2ps")
    return ps


def z2ps(z, zs, plev=PLEV17):
    """Surface pressure [hPa] from geopotential height z (nlat, nlon, nlev)
    [gpm] and surface height zs (nlat, nlon) [m] (basicstate.py:115-151)."""
    return asnumpy(_z2ps_dev(z, zs, plev))


def _spline_dev(x, z, xi, omisb=False, omist=False, xmiss=XMISS):
    x, z, xi = _dev(x), _dev(z), _dev(xi)
    nk, nl = x.numel(), xi.shape[-1]
    ncol = z.numel() // nk
    out = torch.empty(xi.shape, dtype=torch.float64, device=z.device)
    check(lib().lbm_spline(ncol, nk, nl, _p(x), _p(z), _p(xi), _p(out), int(bool(omisb)),
                           int(bool(omist)), float(xmiss), _st()), "lbm_spline")
    return out


def spline(x, z, xi, omisb=False, omist=False, xmiss=XMISS):
    """Natural cubic spline through (x, z[n]) at xi[n] (basicstate.py:176-238):
    x (k,) shared and monotonic, z (n, k), xi (n, l) -> (n, l)."""
    return asnumpy(_spline_dev(x, z, xi, omisb, omist, xmiss))


def _p2s_dev(gdi, ps, sig, plev=PLEV17, xmiss=XMISS):
    g = _dev(gdi)
    lead, nlevp = tuple(g.shape[:-1]), g.shape[-1]
    lnp = torch.log(_dev(plev))
    lns = torch.log(_dev(ps).reshape(-1, 1) * _dev(sig).reshape(1, -1))
    out = _spline_dev(lnp, g.reshape(-1, nlevp), lns, xmiss=xmiss)
    return out.reshape(lead + (-1,))


def p2s(gdi, ps, sig, plev=PLEV17, xmiss=XMISS):
    """Pressure -> sigma levels (basicstate.py:241-260): gdi (nlat, nlon,
    nlevp) on ``plev``, ps (nlat, nlon) [hPa], sig (kmax,).  Leading axes
    beyond (nlat, nlon) -- several basic states at once -- are columns too."""
    return asnumpy(_p2s_dev(gdi, ps, sig, plev, xmiss))


def _zmsw_dev(field, ozm=False, osw=False):
    f = _dev(field).clone()
    if not (ozm or osw):
        return f
    g = f if f.dim() == 3 else f.unsqueeze(-1)
    nlat, nlon, nk = g.shape
    check(lib().lbm_zonal_filter(nlat, nlon, nk, _p(g), 1 if ozm else 2, _st()),
          "lbm_zonal_filter")
    return g if f.dim() == 3 else g[..., 0]


def zmsw(field, ozm=False, osw=False):
    """Zonal mean (``ozm``) or deviation from it (``osw``) along longitude
    (basicstate.py:165-173); unchanged if neither."""
    return asnumpy(_zmsw_dev(field, ozm, osw))


def specsm(field, sp):
    """Spectral smoothing: the model truncation's grid -> wave -> grid round
    trip (basicstate.py:154-162)."""
    return asnumpy(sp.truncate(field))


# ---------------------------------------------------------------------------
# Container and pipeline (basicstate.py:263-324)
# ---------------------------------------------------------------------------
@dataclass
class BasicState:
    """Basic state on the model's sigma levels, north-first Gaussian grid."""

    u: np.ndarray            # (nlat, nlon, kmax) m/s
    v: np.ndarray            # (nlat, nlon, kmax) m/s
    t: np.ndarray            # (nlat, nlon, kmax) K
    q: np.ndarray            # (nlat, nlon, kmax) kg/kg
    ps: np.ndarray           # (nlat, nlon) hPa
    lat_deg: np.ndarray = None
    lon_deg: np.ndarray = None
    sig: np.ndarray = None
    source: str = ""

    def summary(self):
        print(f"basic state from {self.source}")
        print(f"  grid {self.t.shape[0]} lat x {self.t.shape[1]} lon "
              f"x {self.t.shape[2]} sigma levels")
        for name, a, unit in (("u", self.u, "m/s"), ("v", self.v, "m/s"), ("t", self.t, "K"),
                              ("q", self.q, "kg/kg"), ("ps", self.ps, "hPa")):
            print(f"  {name:3s} min {a.min():11.4f}  max {a.max():11.4f}  "
                  f"mean {a.mean():11.4f}   [{unit}]")
        if not all(np.all(np.isfinite(a)) for a in (self.u, self.v, self.t, self.q, self.ps)):
            print("  !! non-finite values present")
        return self


def load_basic_state(path, sp, vgrid, kmo=1, navg=3, zs=None, ozm=False, osw=False,
                     smooth=True, yflip=True, plev=PLEV17):
    """read -> average -> ps from z -> (smooth) -> zonal filter -> p -> sigma
    for u, v, t, q -> (smooth) -> zonal filter.  ps is smoothed before the
    vertical interpolation, u, v, t, q after it (basicstate.py:292-324)."""
    raw = read_pressure_levels(path, kmo=kmo, navg=navg, nlon=sp.nlon, nlat=sp.nlat,
                               nlev=len(plev), yflip=yflip)
    if zs is None:
        zs = np.zeros((sp.nlat, sp.nlon))
    ps = _z2ps_dev(raw["z"], zs, plev)
    if smooth:
        ps = _dev(sp.truncate(ps))
    ps = _zmsw_dev(ps, ozm, osw)
    sig = np.asarray(asnumpy(vgrid.sig), dtype=np.float64)
    out = {}
    for name in ("u", "v", "t", "q"):
        f = _p2s_dev(raw[name], ps, sig, plev)
        if smooth:
            f = _dev(sp.truncate(f))
        out[name] = asnumpy(_zmsw_dev(f, ozm, osw))
    return BasicState(u=out["u"], v=out["v"], t=out["t"], q=out["q"], ps=asnumpy(ps),
                      lat_deg=np.asarray(sp.lat_deg), lon_deg=np.asarray(sp.lon_deg), sig=sig,
                      source=path)
