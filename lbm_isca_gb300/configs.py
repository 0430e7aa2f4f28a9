"""Synthetic inputs for the benchmark workloads (numpy only, host side).

The reference ships no analytic basic-state constructor and its realistic
inputs (ERA5 basic states, MJO forcing files) are not available, so the
workloads are defined here once and consumed unchanged by the GPU path, the
CPU oracle and the bench:

* grid: T21 (64x32), T42 (128x64) or T85 (256x128) Gaussian grid;
  L20/L40 equally spaced pure-sigma half levels ``linspace(1, 0, K+1)``;
* basic state: solid-body zonal flow ``u = 15 cos(lat)`` m/s, ``v = q = 0``,
  temperature ``T(sigma) = max(288 K * sigma**(R*0.0065/g), 216.65 K)``
  (a 6.5 K/km lapse with a stratospheric floor), and surface pressure in
  gradient-wind balance with the solid-body flow about the surface
  temperature, ``ln ps = ln 1000 hPa - a*U0*(2*Omega + U0/a)*sin^2(lat)/(2*R*288)``;
* heating: a compact cos^2 ellipse ``H = cos^2(pi*r/2)`` for ``r < 1`` with
  ``r = sqrt((dlon/30)^2 + (lat/10)^2)`` (degrees) centred on (0N, 120E),
  times ``sin(pi*s(sigma))`` where ``s`` maps [0, sp] -> [0, 1/2] and
  [sp, 1] -> [1/2, 1] piecewise linearly, so the profile peaks at sigma = sp
  (0.45) and vanishes at sigma = 0 and 1; peak 2 K/day, returned in K/s;
* damping of the plain configuration: Rayleigh/Newtonian drag of
  [1, 30 x (K-2), 1] days, del^4 hyperdiffusion with a 6-h e-folding at
  n = N, no sponge, no vertical diffusion, Robert coefficient 0.04,
  dt = 1200 s, two forward start-up calls;
* ensembles: ``numpy.random.default_rng(seed)``; per member, in this order,
  centre longitude ~ U(0, 360), latitude ~ U(-15, 15), amplitude ~
  lognormal(ln 2, 0.5) K/day and peak sigma ~ U(0.3, 0.6).
"""

from __future__ import annotations

import math
import types

import numpy as np

from .constants import ER, GRAV, OMEGA, RAIR

#: truncation -> (nlon, nlat, nmax)
GRIDS = {"T21": (64, 32, 21), "T42": (128, 64, 42), "T85": (256, 128, 85)}

LAPSE_K_PER_M = 0.0065
T_SURFACE = 288.0
T_FLOOR = 216.65
U0_SOLID = 15.0
PS_EQUATOR_HPA = 1000.0


def equal_sigma_half_levels(K):
    """Half-level sigma, index 0 = surface (1.0), index K = top (0.0)."""
    return np.linspace(1.0, 0.0, K + 1)


def full_level_sigma(sigm):
    """Simmons-Burridge full-level sigma for pure-sigma half levels.

    Same formula as the package's ``VerticalGrid.sig``; computed here on the
    host so the synthetic inputs do not need a device.
    """
    sigm = np.asarray(sigm, dtype=np.float64)
    bot, top = sigm[:-1], sigm[1:]
    safe = np.where(top > 0.0, top, 1.0)
    ratio = np.where(top > 0.0, top * (np.log(bot) - np.log(safe)) / (bot - top), 0.0)
    return bot * np.exp(-(1.0 - ratio))


def gaussian_latitudes(nlat):
    """(mu, lat_deg) north first, the same nodes the transforms use."""
    x, _ = np.polynomial.legendre.leggauss(nlat)
    mu = np.sort(x)[::-1]
    return mu, np.degrees(np.arcsin(mu))


def solid_body_basic_state(nlon, nlat, sigm, u0=U0_SOLID, radius=ER):
    """Solid-body basic state (duck-typed like the reference's basic_state)."""
    K = len(sigm) - 1
    mu, _ = gaussian_latitudes(nlat)
    coslat = np.sqrt(1.0 - mu * mu)
    sig = full_level_sigma(sigm)
    expo = RAIR * LAPSE_K_PER_M / GRAV
    tprof = np.maximum(T_SURFACE * sig ** expo, T_FLOOR)
    u = np.broadcast_to((u0 * coslat)[:, None, None], (nlat, nlon, K)).copy()
    v = np.zeros((nlat, nlon, K))
    t = np.broadcast_to(tprof[None, None, :], (nlat, nlon, K)).copy()
    q = np.zeros((nlat, nlon, K))
    coef = radius * u0 * (2.0 * OMEGA + u0 / radius) / (2.0 * RAIR * T_SURFACE)
    lnps = math.log(PS_EQUATOR_HPA) - coef * mu * mu
    ps = np.broadcast_to(np.exp(lnps)[:, None], (nlat, nlon)).copy()
    return types.SimpleNamespace(u=u, v=v, t=t, q=q, ps=ps)


def heating_profile(sig, sigma_peak):
    """sin(pi*s(sigma)) with s piecewise linear, peak exactly at sigma_peak."""
    sig = np.asarray(sig, dtype=np.float64)
    s = np.where(sig <= sigma_peak, 0.5 * sig / sigma_peak,
                 0.5 + 0.5 * (sig - sigma_peak) / (1.0 - sigma_peak))
    return np.sin(np.pi * s)


def elliptic_heating(nlon, nlat, sigm, lon0=120.0, lat0=0.0, amp_k_per_day=2.0,
                     sigma_peak=0.45, half_lon=30.0, half_lat=10.0):
    """Heating in K/s, shape (nlat, nlon, K)."""
    _, lat = gaussian_latitudes(nlat)
    lon = np.arange(nlon) * 360.0 / nlon
    dl = (lon[None, :] - lon0 + 180.0) % 360.0 - 180.0
    r = np.sqrt((dl / half_lon) ** 2 + ((lat[:, None] - lat0) / half_lat) ** 2)
    h = np.where(r < 1.0, np.cos(0.5 * np.pi * r) ** 2, 0.0)
    prof = heating_profile(full_level_sigma(sigm), sigma_peak)
    return h[:, :, None] * prof[None, None, :] * (amp_k_per_day / 86400.0)


def ensemble_heating(nlon, nlat, sigm, nmem, seed):
    """Seeded per-member heatings, shape (nmem, nlat, nlon, K), K/s."""
    rng = np.random.default_rng(seed)
    out = np.empty((nmem, nlat, nlon, len(sigm) - 1))
    params = []
    for e in range(nmem):
        lon0 = rng.uniform(0.0, 360.0)
        lat0 = rng.uniform(-15.0, 15.0)
        amp = rng.lognormal(math.log(2.0), 0.5)
        sp = rng.uniform(0.3, 0.6)
        params.append((lon0, lat0, amp, sp))
        out[e] = elliptic_heating(nlon, nlat, sigm, lon0=lon0, lat0=lat0,
                                  amp_k_per_day=amp, sigma_peak=sp)
    return out, params


def grouped_heating(groups, seed=4):
    """Seeded heatings of an uneven ensemble (the mixed-truncation
    configuration): one generator draws the members of every group in order
    (all of the first group, then the second, ...), each member's centre
    (lon U(0, 360), lat U(-15, 15)), amplitude (lognormal, median 2 K/day,
    sigma 0.5) and peak sigma (U(0.3, 0.6)) as ensemble_heating draws them.
    groups: [(nlon, nlat, sigm, nmem)]; returns a list of (nmem, nlat, nlon,
    K) arrays in K/s."""
    rng = np.random.default_rng(seed)
    out = []
    for nlon, nlat, sigm, nmem in groups:
        h = np.empty((nmem, nlat, nlon, len(sigm) - 1))
        for e in range(nmem):
            lon0 = rng.uniform(0.0, 360.0)
            lat0 = rng.uniform(-15.0, 15.0)
            amp = rng.lognormal(math.log(2.0), 0.5)
            sp = rng.uniform(0.3, 0.6)
            h[e] = elliptic_heating(nlon, nlat, sigm, lon0=lon0, lat0=lat0, amp_k_per_day=amp,
                                    sigma_peak=sp)
        out.append(h)
    return out


def plain_damping(K):
    """Config keywords of the plain configuration's damping."""
    drag = [1.0] + [30.0] * (K - 2) + [1.0]
    return dict(hdif_order=4, hdif_tefold=6.0, hdif_tunit="HOUR", sponge=False,
                ddragv=list(drag), ddragd=list(drag), ddragt=list(drag),
                ddragq=None, vdifv=None, vdifd=None, vdift=None, vdifq=None,
                robert=0.04, delt=1200.0, inistp=2, strictly_linear=False)


def response_box(lat_deg, lon_deg, lat_lo=30.0, lat_hi=60.0, lon_lo=150.0,
                 lon_hi=210.0):
    """Boolean (nlat, nlon) mask of the response-averaging box."""
    la = (lat_deg >= lat_lo) & (lat_deg <= lat_hi)
    lo = (lon_deg >= lon_lo) & (lon_deg <= lon_hi)
    return la[:, None] & lo[None, :]
