"""Seeded inputs of the format and setup fixtures (``make_golden_io.py``) and
of the tests that compare against them: history fields, geopotential-height
columns, spline cases, a synthetic ERA5-like pressure-level file, fields to
regrid.  Nothing here depends on the reference or on a GPU."""

import numpy as np

PLEV17 = np.array([1000., 925., 850., 700., 600., 500., 400., 300., 250.,
                   200., 150., 100., 70., 50., 30., 20., 10.])
SIGM5 = np.array([1.0, 0.85, 0.6, 0.35, 0.15, 0.0])      # 5 sigma layers
UNDEF_IN = -9.999e20


def lat_deg(nlat):
    return np.linspace(80.0, -80.0, nlat)


def history_days(nlat, nlon, kmax, ndays, seed=3):
    rng = np.random.default_rng(seed)
    scale = {"psi": 1e7, "chi": 1e6, "u": 10.0, "v": 5.0, "w": 1e-3, "t": 2.0, "z": 50.0}
    days = []
    for _ in range(ndays):
        f = {k: rng.standard_normal((nlat, nlon, kmax)) * s for k, s in scale.items()}
        f["p"] = rng.standard_normal((nlat, nlon)) * 3.0
        days.append(f)
    return days


def _z_profile(rng, n, plev, z0_spread=60.0):
    """Heights increasing with the level index (pressure decreasing)."""
    base = 7300.0 * np.log(1000.0 / plev)
    return base[None, :] + rng.standard_normal((n, 1)) * z0_spread + \
        np.cumsum(np.abs(rng.standard_normal((n, plev.size))) * 5.0, axis=1)


def heights(ncol, seed=1):
    rng = np.random.default_rng(seed)
    z = _z_profile(rng, ncol, PLEV17)
    zs = rng.uniform(-200.0, 3500.0, ncol)
    zs[0] = z[0, 0] - 50.0          # below the lowest level
    zs[1] = z[1, -1] + 100.0        # above the top level
    zs[2] = z[2, 3]                 # exactly on a level
    return z, zs


def spline_case(ncol, nl=9, seed=2):
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((ncol, PLEV17.size)).cumsum(axis=1) * 3.0 + 250.0
    p = np.exp(rng.uniform(np.log(4.0), np.log(1100.0), (ncol, nl)))
    p[0, 0], p[1, 0] = 1050.0, 8.0    # beyond both ends
    p[2, 0] = PLEV17[5]               # exactly on a level
    return z, np.log(p)


def p2s_case(seed=4):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((4, 8, PLEV17.size)).cumsum(axis=-1) + 280.0
    ps = rng.uniform(500.0, 1040.0, (4, 8))
    sig = np.array([0.995, 0.9, 0.7, 0.4, 0.05])
    return g, ps, sig


def zonal_case(seed=6):
    return np.random.default_rng(seed).standard_normal((4, 8, 3)) * 7.0 + 3.0


def write_pressure_file(path, nlon, nlat, nlev, nmonth, seed, undef=False):
    """Fortran sequential big-endian real*4 records, (nlon, nlat) each, rows
    south first, ordered month -> variable (z, rhum, q, t, u, v, omega) ->
    level; with ``undef`` a few points of the first month hold the input
    files' undefined value (as real*4)."""
    rng = np.random.default_rng(seed)
    plev = PLEV17[:nlev] if nlev <= PLEV17.size else np.linspace(1000.0, 10.0, nlev)
    lat = np.radians(np.linspace(-85.0, 85.0, nlat))[:, None]
    lon = np.radians(np.arange(nlon) * 360.0 / nlon)[None, :]
    recs = []
    for mo in range(nmonth):
        zc = _z_profile(rng, 1, plev, 30.0)[0]
        for var in range(7):
            for k in range(nlev):
                if var == 0:
                    f = zc[k] + 80.0 * np.cos(lat) * np.cos(lon + 0.3 * mo) + \
                        rng.standard_normal((nlat, nlon)) * 4.0
                elif var == 2:
                    f = 1e-3 * np.exp(-k / 4.0) * (1.0 + 0.3 * np.cos(lat) * np.sin(2 * lon))
                elif var == 3:
                    f = 290.0 - 40.0 * k / nlev - 20.0 * np.sin(lat) ** 2 + \
                        rng.standard_normal((nlat, nlon))
                elif var == 4:
                    f = 20.0 * np.cos(lat) ** 2 * (1.0 + k / nlev) + 2.0 * np.sin(lon - mo)
                elif var == 5:
                    f = 3.0 * np.sin(2 * lat) * np.cos(3 * lon + k)
                else:
                    f = rng.standard_normal((nlat, nlon))
                f = np.asarray(f, dtype=np.float64) * np.ones((nlat, nlon))
                if undef and var in (3, 4) and mo == 0:
                    f[1, 2] = UNDEF_IN
                recs.append(f)
    npts = nlon * nlat
    with open(path, "wb") as fh:
        for f in recs:
            marker = np.array([npts * 4], dtype=">i4")
            marker.tofile(fh)
            np.ascontiguousarray(f, dtype=">f4").tofile(fh)
            marker.tofile(fh)
    return plev


def regrid_fields(lat_deg_arr, nlon=64):
    lat = np.radians(np.asarray(lat_deg_arr))[:, None]
    lon = np.radians(np.arange(nlon) * 360.0 / nlon)[None, :]
    s2 = np.cos(lat) ** 2 * np.cos(3 * lon) + 0.5 * np.sin(lat) ** 3 + 0.2 * np.cos(lat) * np.sin(14 * lon)
    s3 = np.stack([s2 * 2.0 + 1.0, np.sin(lat) * np.cos(lat) ** 5 * np.sin(7 * lon)], axis=-1)
    u = 20.0 * np.cos(lat) ** 2 + 3.0 * np.cos(lat) * np.sin(2 * lon) * np.sin(lat)
    v = 4.0 * np.cos(lat) * np.cos(5 * lon) * np.sin(lat)
    return s2, s3, u, v
