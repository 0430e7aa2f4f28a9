"""CPU oracle for the PyLBM-Isca dynamical-core hot path.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the GB300 kernels
are compared against, and the CPU baseline that ``bench.py`` times.  It is a
plain-numpy restatement of the reference algorithm (kuiper2000/LBM_isca,
``pylbm_isca``), written independently and following the reference's
formulas step for step so that it reproduces the reference to round-off.
Nothing in the product package imports it; only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (cpu baseline / reference arm)
may.

Pinning: ``tests/test_oracle_golden.py`` compares every public quantity here
against vectors produced by running the reference itself
(``tests/golden/make_golden.py``), and against the numbers the reference
records in ``analysis/gill_isca.json``.

Conventions (same as the reference):
* grid fields ``(..., nlat, nlon[, K])``, latitudes north -> south;
* spectral fields ``(..., M, M[, K])`` complex, indexed ``[m, n]``, zero for
  ``n < m`` (M = nmax + 1);
* levels bottom-up (k = 0 is the lowest layer).

Third-party arithmetic used here (present in this image, pinned only by the
reference's lower bounds numpy>=1.24): ``numpy.polynomial.legendre.leggauss``
for the Gauss nodes (spectral.py:58), ``numpy.fft.rfft/irfft`` (pocketfft)
for the longitude transforms (spectral.py:159-172), ``matmul``/``einsum`` and
``linalg.inv`` (integrator.py:161, 226).
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

# --------------------------------------------------------------------------
# Physical constants -- values of constants.py:38-56 (GFDL/Isca defaults).
# --------------------------------------------------------------------------
EARTH_RADIUS = 6.371e6
GRAVITY = 9.80
R_DRY = 287.04
R_VAP = 461.50
KAPPA = 2.0 / 7.0
OMEGA = 7.2921150e-5
EPS_VIRT = R_VAP / R_DRY - 1.0
SEC_PER_DAY = 86400.0

# L20 half levels of constants.py:92-97 (index 0 = surface).
SIGMA_HALF_L20 = np.array([1.000, 0.990, 0.970, 0.930, 0.870, 0.790, 0.700,
                           0.600, 0.500, 0.410, 0.330, 0.260, 0.200, 0.150,
                           0.100, 0.070, 0.050, 0.040, 0.030, 0.020, 0.000])

# &nmdamp default profile of model.py:30-31, in days.
DRAG_DAYS_DEFAULT = [0.5, 0.5, 0.5, 5, 15] + [20] * 13 + [0.5, 0.5]


def time_unit_seconds(value, unit):
    """integrator.py:115-118: value in SEC/MIN/HOUR/DAY/MONth -> seconds."""
    scale = {"SEC": 1.0, "MIN": 60.0, "HOU": 3600.0, "DAY": SEC_PER_DAY,
             "MON": 30.0 * SEC_PER_DAY}
    return float(value) * scale[unit.strip().upper()[:3]]


# ==========================================================================
# Spherical-harmonic transforms  (spectral.py)
# ==========================================================================
class SphericalTransform:
    """Gaussian grid + transforms, restating spectral.py:49-281."""

    def __init__(self, nlon=128, nlat=64, nmax=42, radius=EARTH_RADIUS):
        self.nlon, self.nlat, self.nmax = int(nlon), int(nlat), int(nmax)
        self.a = float(radius)
        M = self.nmax + 1
        # spectral.py:58-61 -- nodes sorted north first, weights summing to 1
        x, w = np.polynomial.legendre.leggauss(self.nlat)
        idx = np.argsort(-x)
        self.mu = x[idx]
        self.gw = 0.5 * w[idx]
        self.coslat = np.sqrt(1.0 - self.mu ** 2)
        self.lat = np.arcsin(self.mu)
        self.lon = 2.0 * np.pi * np.arange(self.nlon) / self.nlon
        # spectral.py:68
        self.gwdel = self.gw / (self.a * (1.0 - self.mu ** 2))
        self.P, self.H, self.eps = legendre_tables(self.nmax, self.mu)
        n = np.arange(M, dtype=np.float64)
        self.nn1 = n * (n + 1.0)
        self.lap = -self.nn1 / self.a ** 2                      # spectral.py:76
        self.invlap = np.zeros(M)
        self.invlap[1:] = -self.a ** 2 / self.nn1[1:]            # spectral.py:78
        self.im = 1j * np.arange(M, dtype=np.float64)            # spectral.py:84
        mm, nn = np.meshgrid(np.arange(M), np.arange(M), indexing="ij")
        self.mask = nn >= mm                                     # spectral.py:88-90
        # pre-weighted tables, spectral.py:149-154
        self.P_gw = self.P * self.gw
        self.P_gwdel = self.P * self.gwdel
        self.H_gwdel = self.H * self.gwdel
        self.PT = np.ascontiguousarray(np.swapaxes(self.P, 1, 2))
        self.HT = np.ascontiguousarray(np.swapaxes(self.H, 1, 2))

    #: True when arrays carry a leading member axis (ensemble.py:41-72)
    batched = False

    def batched_view(self):
        """The same transform with a leading member axis on every array."""
        other = object.__new__(type(self))
        other.__dict__.update(self.__dict__)
        other.batched = True
        return other

    def _has_k(self, x):
        return np.ndim(x) == (4 if self.batched else 3)

    # ---- layout helpers: collapse leading/level axes into columns ---------
    def _to_cols_grid(self, f, has_k):
        f = np.asarray(f, dtype=np.float64)
        lead = f.shape[:-3] if has_k else f.shape[:-2]
        J, I = self.nlat, self.nlon
        if has_k:
            K = f.shape[-1]
            g = np.moveaxis(f.reshape((-1, J, I, K)), 0, 2).reshape(J, I, -1)
        else:
            K = None
            g = np.moveaxis(f.reshape((-1, J, I)), 0, 2)
        return g, (lead, K)

    def _from_cols_grid(self, g, meta):
        lead, K = meta
        J, I = g.shape[:2]
        if K is None:
            return np.moveaxis(g, 2, 0).reshape(lead + (J, I))
        return np.moveaxis(g.reshape(J, I, -1, K), 2, 0).reshape(lead + (J, I, K))

    def _to_cols_spec(self, x, has_k):
        x = np.asarray(x)
        M = self.nmax + 1
        lead = x.shape[:-3] if has_k else x.shape[:-2]
        if has_k:
            K = x.shape[-1]
            s = np.moveaxis(x.reshape((-1, M, M, K)), 0, 2).reshape(M, M, -1)
        else:
            K = None
            s = np.moveaxis(x.reshape((-1, M, M)), 0, 2)
        return s.astype(np.complex128), (lead, K)

    _from_cols_spec = _from_cols_grid

    # ---- Fourier, spectral.py:159-172 -------------------------------------
    def fourier_fwd(self, g):
        """(J, I, C) real -> (M, J, C) complex, rfft/nlon truncated to m<=N."""
        F = np.fft.rfft(g, axis=1)[:, :self.nmax + 1] / self.nlon
        return np.ascontiguousarray(np.moveaxis(F, 1, 0))

    def fourier_inv(self, F):
        """(M, J, C) complex -> (J, I, C) real; m=0 imaginary part dropped."""
        M, J, C = F.shape
        full = np.zeros((J, self.nlon // 2 + 1, C), dtype=np.complex128)
        full[:, :M] = np.moveaxis(F, 0, 1)
        return np.fft.irfft(full * self.nlon, n=self.nlon, axis=1)

    # ---- scalar transforms, spectral.py:186-197 ----------------------------
    def grid_to_wave(self, f):
        g, meta = self._to_cols_grid(f, self._has_k(f))
        xi = np.matmul(self.P_gw, self.fourier_fwd(g))
        return self._from_cols_spec(xi, meta)

    def wave_to_grid(self, x):
        s, meta = self._to_cols_spec(x, self._has_k(x))
        g = self.fourier_inv(np.matmul(self.PT, s))
        return self._from_cols_grid(g, meta)

    # ---- operators, spectral.py:202-276 -------------------------------------
    def _nfac(self, x, v):
        x = np.asarray(x)
        return x * (v[:, None] if self._has_k(x) else v)

    def laplacian(self, x):
        return self._nfac(x, self.lap)

    def inverse_laplacian(self, x):
        return self._nfac(x, self.invlap)

    def hgrad(self, x):
        """spectral.py:210-225: grid (d/dx, d/dy) of a spectral scalar."""
        s, meta = self._to_cols_spec(x, self._has_k(x))
        scale = (1.0 / (self.a * self.coslat))[:, None, None]
        gx = self.fourier_inv(np.matmul(self.PT, self.im[:, None, None] * s)) * scale
        gy = self.fourier_inv(np.matmul(self.HT, s)) * scale
        return self._from_cols_grid(gx, meta), self._from_cols_grid(gy, meta)

    def uv_to_vordiv(self, u, v):
        """spectral.py:227-244."""
        has_k = self._has_k(u)
        gu, meta = self._to_cols_grid(u, has_k)
        gv, _ = self._to_cols_grid(v, has_k)
        c = self.coslat[:, None, None]
        Fu = self.fourier_fwd(gu * c)
        Fv = self.fourier_fwd(gv * c)
        im = self.im[:, None, None]
        vor = np.matmul(self.P_gwdel, im * Fv) + np.matmul(self.H_gwdel, Fu)
        div = np.matmul(self.P_gwdel, im * Fu) - np.matmul(self.H_gwdel, Fv)
        return self._from_cols_spec(vor, meta), self._from_cols_spec(div, meta)

    def neg_divergence(self, fx, fy):
        return -self.uv_to_vordiv(fx, fy)[1]

    def curl(self, fx, fy):
        return self.uv_to_vordiv(fx, fy)[0]

    def psichi_to_uv(self, psi, chi):
        """spectral.py:262-276."""
        has_k = self._has_k(psi)
        sp, meta = self._to_cols_spec(psi, has_k)
        sc, _ = self._to_cols_spec(chi, has_k)
        im = self.im[:, None, None]
        Um = np.matmul(self.PT, im * sc) - np.matmul(self.HT, sp)
        Vm = np.matmul(self.PT, im * sp) + np.matmul(self.HT, sc)
        scale = (1.0 / (self.a * self.coslat))[:, None, None]
        u = self.fourier_inv(Um) * scale
        v = self.fourier_inv(Vm) * scale
        return self._from_cols_grid(u, meta), self._from_cols_grid(v, meta)

    def vordiv_to_uv(self, vor, div):
        return self.psichi_to_uv(self.inverse_laplacian(vor),
                                 self.inverse_laplacian(div))

    def truncate(self, f):
        return self.wave_to_grid(self.grid_to_wave(f))


def legendre_tables(nmax, mu):
    """Fully normalised P_n^m(mu) (no Condon-Shortley phase, (1/2)int P^2 = 1)
    and H_n^m = (1-mu^2) dP_n^m/dmu, following spectral.py:102-141.

    Returns P[m, n, j] and H[m, n, j] for 0 <= m, n <= nmax (zero for n < m)
    and eps[m, n] = sqrt((n^2-m^2)/(4n^2-1)) for n <= nmax+1.
    """
    M = nmax + 1
    nx = nmax + 2
    J = mu.size
    s = np.sqrt(1.0 - mu * mu)
    n = np.arange(nx, dtype=np.float64)
    eps = np.zeros((M, nx))
    for m in range(M):
        k = n[m + 1:]
        eps[m, m + 1:] = np.sqrt((k * k - m * m) / (4.0 * k * k - 1.0))
    P = np.zeros((M, nx, J))
    diag = np.ones(J)
    for m in range(M):
        if m > 0:                                    # spectral.py:118-119
            diag = diag * math.sqrt((2.0 * m + 1.0) / (2.0 * m)) * s
        P[m, m] = diag
        P[m, m + 1] = diag * math.sqrt(2.0 * m + 3.0) * mu   # spectral.py:123
        for k in range(m + 2, nx):                   # spectral.py:125-128
            P[m, k] = (mu * P[m, k - 1] - eps[m, k - 1] * P[m, k - 2]) / eps[m, k]
    H = np.zeros((M, M, J))
    for m in range(M):                               # spectral.py:133-138
        for k in range(m, M):
            h = -k * eps[m, k + 1] * P[m, k + 1]
            if k - 1 >= m:
                h = h + (k + 1.0) * eps[m, k] * P[m, k - 1]
            H[m, k] = h
    return np.ascontiguousarray(P[:, :M]), H, eps


# ==========================================================================
# Simmons-Burridge vertical operators  (vertical.py)
# ==========================================================================
class SigmaLevels:
    """Restates VerticalGrid (vertical.py:59-203) and compute_tbar (206-216)."""

    def __init__(self, sigm=SIGMA_HALF_L20, kappa=KAPPA):
        sigm = np.asarray(sigm, dtype=np.float64)
        self.sigm = sigm
        self.kmax = K = sigm.size - 1
        self.kappa = kappa
        bot, top = sigm[:-1], sigm[1:]
        self.dsig = bot - top
        safe_top = np.where(top > 0.0, top, 1.0)
        lr = np.log(bot) - np.log(safe_top)
        # vertical.py:343-347: alpha, with alpha=1 in the massless top layer
        self.alpha = 1.0 - np.where(top > 0.0, top * lr / (bot - top), 0.0)
        self.sig = bot * np.exp(-self.alpha)                 # vertical.py:350
        self.dlog1 = self.alpha.copy()
        self.dlog2 = np.where(top > 0.0, np.log(self.sig) - np.log(safe_top), 0.0)
        self.dlog3 = np.where(top > 0.0, lr, 0.0)
        self.cpg = (bot * self.dlog1 + top * self.dlog2) / self.dsig   # :368
        self.w3 = self.dlog3 / self.dsig                              # :373
        self.wP = self.alpha - self.cpg                               # :374
        dsm = np.empty(K + 1)                                         # :377-380
        dsm[0] = sigm[0] - self.sig[0]
        dsm[1:K] = self.sig[:-1] - self.sig[1:]
        dsm[K] = self.sig[-1] - sigm[-1]
        self.dsigm = dsm
        ww = np.tril(np.ones((K, K)), -1) * (R_DRY * self.dlog3)[None, :]
        ww[np.arange(K), np.arange(K)] = R_DRY * self.alpha           # :384-391
        self.ww = ww
        self.tbar = self.gg = self.tmtx = self.whmtx = self.gcmtx = None

    def set_reference_temperature(self, tbar):
        """vertical.py:440-462."""
        K = self.kmax
        tbar = np.array(tbar, dtype=np.float64)
        self.tbar = tbar
        self.gg = R_DRY * tbar * self.cpg
        above = np.triu(np.ones((K, K)), 1) * self.dsig[None, :]
        tm = KAPPA * tbar[:, None] * self.w3[:, None] * above
        tm[np.arange(K), np.arange(K)] = KAPPA * tbar * self.alpha
        self.tmtx = tm
        self.whmtx = self.ww @ tm
        self.gcmtx = np.outer(self.gg, self.dsig)

    def hydrostatic(self, tv):
        return np.asarray(tv) @ self.ww.T


def compute_tbar(tv):
    """vertical.py:206-216: plain mean over the (nlat, nlon) grid."""
    tv = np.asarray(tv)
    return tv.sum(axis=(0, 1)) / (tv.shape[0] * tv.shape[1])


# ==========================================================================
# Implicit operators  (integrator.py)
# ==========================================================================
def drag_profile(days, K, unit):
    """integrator.py:101-112."""
    out = np.zeros(K)
    if days is None:
        return out
    d = np.asarray(days, dtype=np.float64)
    if d.size != K:
        raise ValueError(f"damping profile must have {K} entries")
    sec = np.array([time_unit_seconds(x, unit) for x in d])
    ok = sec > 0
    out[ok] = 1.0 / sec[ok]
    return out


class DampingCoefs:
    """(n, k) implicit damping coefficients, integrator.py:41-98."""

    def __init__(self, nmax, levels, order=4, tefold=2.0, tunit_hdif="HOUR",
                 ddragv=None, ddragd=None, ddragt=None, ddragq=None,
                 tunit_damp="DAY", ray0=30.0, zsclh=8.0e3, rzsclh=7.0e3,
                 sponge=True):
        K = levels.kmax
        n = np.arange(nmax + 1, dtype=np.float64)
        p = order // 2
        tau = time_unit_seconds(tefold, tunit_hdif)
        ref = (nmax * (nmax + 1.0) / nmax) ** p
        dt_n = (n * (n + 1.0) / nmax) ** p
        dv_n = dt_n - (2.0 / nmax) ** p
        kt = dt_n / ref / tau
        kv = dv_n / ref / tau
        kt[0] = 0.0
        kv[0] = 0.0
        kv[1] = max(kv[1], 0.0)
        self.kt_h, self.kv_h = kt, kv
        sponge_k = np.zeros(K)
        if sponge:                                    # integrator.py:71-77
            r0 = time_unit_seconds(ray0, tunit_hdif)
            z = -zsclh * np.log(levels.sig)
            ztop = -zsclh * np.log(float(levels.sig[-1]))
            sponge_k = np.maximum(1.0 + np.tanh((z - ztop) / rzsclh), 1e-20) / r0
        self.sponge_k = sponge_k
        dv = drag_profile(ddragv, K, tunit_damp)
        dd = drag_profile(ddragd, K, tunit_damp)
        dtt = drag_profile(ddragt, K, tunit_damp)
        dq = drag_profile(ddragq, K, tunit_damp)
        self.kv = kv[:, None] + (sponge_k + dv)[None, :]
        self.kd = kv[:, None] + (sponge_k + dd)[None, :]
        self.ktt = kt[:, None] + dtt[None, :]
        self.kq = kt[:, None] + dq[None, :]


def gravity_wave_matrices(dt, lap, ktt, kd, whmtx, gcmtx):
    """M(n) = diag(fd*ft) - dt^2 lap(n) (whmtx + gcmtx*ft), integrator.py:149-158."""
    Mn, K = ktt.shape
    out = np.empty((Mn, K, K))
    for n in range(Mn):
        ft = 1.0 + 2.0 * dt * ktt[n]
        fd = 1.0 + 2.0 * dt * kd[n]
        mat = -(dt * dt * lap[n]) * (whmtx + gcmtx * ft[:, None])
        mat[np.arange(K), np.arange(K)] += fd * ft
        out[n] = mat
    return out


def vdiff_operator(levels):
    """Tridiagonal sigma Laplacian with zero-flux ends, integrator.py:182-206."""
    K = levels.kmax
    ds, dsm = levels.dsig, levels.dsigm
    lo = np.zeros(K)
    up = np.zeros(K)
    lo[1:] = 1.0 / (ds[1:] * dsm[1:K])
    up[:-1] = 1.0 / (ds[:-1] * dsm[1:K])
    di = -(lo + up)
    up[0] = (dsm[0] + dsm[1]) / (ds[0] * dsm[0] * dsm[1])
    lo[0] = 0.0
    di[0] = -up[0]
    lo[-1] = (dsm[K - 1] + dsm[K]) / (ds[-1] * dsm[K - 1] * dsm[K])
    up[-1] = 0.0
    di[-1] = -lo[-1]
    L = np.diag(di) + np.diag(lo[1:], -1) + np.diag(up[:-1], 1)
    return L


def vdiff_coef(v, K):
    """integrator.py:243-253."""
    if v is None:
        return None
    v = np.atleast_1d(np.asarray(v, dtype=np.float64))
    if v.size == 1:
        v = np.full(K, v[0])
    if np.any(v <= 0):
        return None
    return 1.0 / (SEC_PER_DAY * v)


# ==========================================================================
# Linearised tendencies  (dynamics.py)
# ==========================================================================
def column_sum(x, dsig):
    """dynamics.py:96-102: S[k] = sum_{l>=k} dsig_l x_l, S[K] = 0."""
    w = x * dsig
    out = np.zeros(x.shape[:-1] + (x.shape[-1] + 1,))
    out[..., :-1] = np.cumsum(w[..., ::-1], axis=-1)[..., ::-1]
    return out


def sigma_dot(S, sigm):
    """dynamics.py:105-114."""
    sd = sigm * S[..., :1] - S
    sd[..., 0] = 0.0
    sd[..., -1] = 0.0
    return sd


def vert_advect(f, sdot, dsig):
    """dynamics.py:117-143 (SECOND_CENTERED, ADVECTIVE_FORM, overall + sign)."""
    K = f.shape[-1]
    lead = np.broadcast_shapes(f.shape[:-1], sdot.shape[:-1])
    flux = np.zeros(lead + (K + 1,))
    flux[..., 1:K] = 0.5 * sdot[..., 1:K] * (f[..., 1:K] + f[..., :K - 1])
    return (flux[..., 1:] - flux[..., :-1] - f * np.diff(sdot, axis=-1)) / dsig


class BasicTerms:
    """Basic-state derived fields, dynamics.py:54-93."""

    def __init__(self, tr, lv, bs):
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
        self.u, self.v, self.t = f64(bs.u), f64(bs.v), f64(bs.t)
        self.q, self.ps = f64(bs.q), f64(bs.ps)
        self.coriol = (2.0 * OMEGA * tr.mu)[:, None]
        self.vor, self.div_s = tr.uv_to_vordiv(self.u, self.v)
        self.vor_g = tr.wave_to_grid(self.vor)
        self.div = tr.wave_to_grid(self.div_s)
        self.lnps = np.log(self.ps)
        self.pix, self.piy = tr.hgrad(tr.grid_to_wave(self.lnps))
        self.tv = self.t * (1.0 + EPS_VIRT * self.q)
        self.padv = self.u * self.pix[..., None] + self.v * self.piy[..., None]
        self.ssum = column_sum(self.div + self.padv, lv.dsig)
        self.sdot = sigma_dot(self.ssum, lv.sigm)
        self.x5 = lv.w3 * self.ssum[..., 1:] + lv.alpha * self.div + lv.wP * self.padv
        lv.set_reference_temperature(compute_tbar(self.tv))


def tendencies(tr, lv, bt, st, frc_t=None, frc_vor=None, frc_div=None,
               frc_ps=None, frc_q=None, strictly_linear=False, diag=None):
    """Explicit spectral tendencies (vor, div, T, pi, q), dynamics.py:156-271.

    ``st`` carries grid u, v, t, q (..., J, I, K), ps (..., J, I) and ps_bar.
    """
    ds, sm = lv.dsig, lv.sigm
    tref = lv.tbar
    up, vp, tp, qp = st.u, st.v, st.t, st.q
    vor_s, div_s = tr.uv_to_vordiv(up, vp)
    vor = tr.wave_to_grid(vor_s)
    div = tr.wave_to_grid(div_s)
    pi = np.log(st.ps_bar + st.ps) - np.log(st.ps_bar)
    pix, piy = tr.hgrad(tr.grid_to_wave(pi))
    pad = (up * bt.pix[..., None] + bt.u * pix[..., None]
           + vp * bt.piy[..., None] + bt.v * piy[..., None])
    S = column_sum(div + pad, ds)
    sd = sigma_dot(S, sm)
    tv = tp + EPS_VIRT * (tp * bt.q + bt.t * qp)
    # 1. continuity (dynamics.py:188-191)
    gt_pi = -S[..., 0] + (div * ds).sum(axis=-1)
    if frc_ps is not None:
        gt_pi = gt_pi + frc_ps
    wt_pi = tr.grid_to_wave(gt_pi)
    # 2. temperature (dynamics.py:197-219)
    x5p = lv.alpha * div + lv.wP * pad + lv.w3 * S[..., 1:]
    adiab = -KAPPA * (tv * bt.x5 + bt.tv * x5p)
    tdev = bt.t - tref
    xu = up * tdev + bt.u * tp
    xv = vp * tdev + bt.v * tp
    hadv = tp * bt.div + tdev * div
    vadv = vert_advect(tp, bt.sdot, ds) + vert_advect(bt.t, sd, ds)
    gt_t = adiab + hadv + vadv + div @ lv.tmtx.T
    if frc_t is not None:
        gt_t = gt_t + frc_t
    wt_t = tr.neg_divergence(xu, xv) + tr.grid_to_wave(gt_t)
    # 3. momentum (dynamics.py:224-251)
    absvor = bt.vor_g + bt.coriol[..., None]
    fu = vp * absvor + bt.v * vor
    fv = -up * absvor - bt.u * vor
    rcpg = R_DRY * lv.cpg
    tvdev = bt.tv - tref
    fu = fu - rcpg * (tv * bt.pix[..., None] + tvdev * pix[..., None])
    fv = fv - rcpg * (tv * bt.piy[..., None] + tvdev * piy[..., None])
    fu = fu + vert_advect(up, bt.sdot, ds) + vert_advect(bt.u, sd, ds)
    fv = fv + vert_advect(vp, bt.sdot, ds) + vert_advect(bt.v, sd, ds)
    ke = lv.hydrostatic(tv - tp) + up * bt.u + vp * bt.v
    if not strictly_linear:
        ke = ke + 0.5 * (up * up + vp * vp)
    wt_vor, wt_div = tr.uv_to_vordiv(fu, fv)
    wt_div = wt_div - tr.laplacian(tr.grid_to_wave(ke))
    if frc_vor is not None:
        wt_vor = wt_vor + tr.grid_to_wave(frc_vor)
    if frc_div is not None:
        wt_div = wt_div + tr.grid_to_wave(frc_div)
    # 4. humidity (dynamics.py:256-262)
    yu = up * bt.q + bt.u * qp
    yv = vp * bt.q + bt.v * qp
    g = (qp * bt.div + bt.q * div + vert_advect(qp, bt.sdot, ds)
         + vert_advect(bt.q, sd, ds))
    if frc_q is not None:
        g = g + frc_q
    wt_q = tr.neg_divergence(yu, yv) + tr.grid_to_wave(g)
    if diag is not None:          # dynamics.py:267-270
        diag.update(vor=vor, div=div, vor_s=vor_s, div_s=div_s, sdot=sd, pi=pi,
                    omega=-lv.sig * (x5p * bt.ps[..., None]
                                     + bt.x5 * st.ps[..., None]))
    return wt_vor, wt_div, wt_t, wt_pi, wt_q


# ==========================================================================
# State, integrator and time loop  (state.py, integrator.py, model.py)
# ==========================================================================
@dataclasses.dataclass
class GridState:
    """Grid-space perturbation (state.py:26-148); ps in hPa like ps_bar."""
    ps_bar: np.ndarray
    u: np.ndarray
    v: np.ndarray
    t: np.ndarray
    q: np.ndarray
    ps: np.ndarray

    @classmethod
    def zeros(cls, ps_bar, K, nmem=None):
        J, I = ps_bar.shape
        lead = () if nmem is None else (nmem,)
        z = lambda: np.zeros(lead + (J, I, K))    # noqa: E731
        return cls(ps_bar, z(), z(), z(), z(), np.zeros(lead + (J, I)))

    def copy(self):
        return GridState(self.ps_bar, self.u.copy(), self.v.copy(),
                         self.t.copy(), self.q.copy(), self.ps.copy())

    def lnps_pert(self):
        return np.log(self.ps_bar + self.ps) - np.log(self.ps_bar)

    def to_spectral(self, tr):
        """state.py:86-92."""
        vor, div = tr.uv_to_vordiv(self.u, self.v)
        return {"vor": vor, "div": div, "t": tr.grid_to_wave(self.t),
                "pi": tr.grid_to_wave(self.lnps_pert()),
                "q": tr.grid_to_wave(self.q)}

    @classmethod
    def from_spectral(cls, tr, ps_bar, spec):
        """state.py:94-99."""
        u, v = tr.vordiv_to_uv(spec["vor"], spec["div"])
        ps = ps_bar * (np.exp(tr.wave_to_grid(spec["pi"])) - 1.0)
        return cls(ps_bar, u, v, tr.wave_to_grid(spec["t"]),
                   tr.wave_to_grid(spec["q"]), ps)

    def filtered(self, cur, new, gamma):
        """Robert-Asselin on u, v, t, q, ps: self is t-dt (state.py:110-128)."""
        f = lambda p, c, n: c + gamma * (p - 2.0 * c + n)   # noqa: E731
        return GridState(self.ps_bar, f(self.u, cur.u, new.u), f(self.v, cur.v, new.v),
                         f(self.t, cur.t, new.t), f(self.q, cur.q, new.q),
                         f(self.ps, cur.ps, new.ps))

    def isfinite(self):
        return all(np.isfinite(a).all() for a in (self.u, self.v, self.t, self.q, self.ps))


@dataclasses.dataclass
class RunConfig:
    """model.py:34-86 knobs with the reference defaults."""
    delt: float = 1200.0
    inistp: int = 2
    ndays: float = 66.0
    hdif_order: int = 4
    hdif_tefold: float = 2.0
    hdif_tunit: str = "HOUR"
    sponge: bool = True
    ray0: float = 30.0
    ddragv: list = dataclasses.field(default_factory=lambda: list(DRAG_DAYS_DEFAULT))
    ddragd: list = dataclasses.field(default_factory=lambda: list(DRAG_DAYS_DEFAULT))
    ddragt: list = dataclasses.field(default_factory=lambda: list(DRAG_DAYS_DEFAULT))
    ddragq: list = None
    damp_tunit: str = "DAY"
    vdifv: float = 1.0e3
    vdifd: float = 1.0e3
    vdift: float = 1.0e3
    vdifq: float = None
    robert: float = 0.04
    strictly_linear: bool = False

    @property
    def steps_per_day(self):
        return int(round(SEC_PER_DAY / self.delt))


class OracleModel:
    """The reference time loop (model.py:92-290) without history output.

    ``nmem`` adds a leading member axis to the state (ensemble.py:152-165);
    every member shares the basic state and the operators.
    """

    def __init__(self, tr, lv, basic_state, cfg=None, nmem=None):
        self.tr = tr if nmem is None else tr.batched_view()
        self.lv = lv
        self.cfg = c = cfg or RunConfig()
        self.bt = BasicTerms(tr, lv, basic_state)
        self.damp = DampingCoefs(tr.nmax, lv, order=c.hdif_order,
                                 tefold=c.hdif_tefold, tunit_hdif=c.hdif_tunit,
                                 ddragv=c.ddragv, ddragd=c.ddragd,
                                 ddragt=c.ddragt, ddragq=c.ddragq,
                                 tunit_damp=c.damp_tunit, ray0=c.ray0,
                                 sponge=c.sponge)
        K = lv.kmax
        self.vlap = vdiff_operator(lv)
        self.vcoef = {"vor": vdiff_coef(c.vdifv, K), "div": vdiff_coef(c.vdifd, K),
                      "t": vdiff_coef(c.vdift, K), "q": vdiff_coef(c.vdifq, K)}
        self._ops_dt = None
        ps_bar = np.asarray(basic_state.ps, dtype=np.float64)
        self.ga = GridState.zeros(ps_bar, K, nmem)
        self.gb = GridState.zeros(ps_bar, K, nmem)
        self.time = 0.0
        self.istep = 0       # calls of step(), start-up calls included
        self.advanced = 0

    def set_initial_perturbation(self, **fields):
        for k, val in fields.items():
            if val is not None:
                setattr(self.ga, k, np.array(val, dtype=np.float64))
                setattr(self.gb, k, np.array(val, dtype=np.float64))

    def prepare(self, dt):
        """SemiImplicit.prepare + VerticalDiffusion.prepare for this dt."""
        if self._ops_dt == dt:
            return
        d, lv = self.damp, self.lv
        self.gw_mat = gravity_wave_matrices(dt, self.tr.lap, d.ktt, d.kd,
                                            lv.whmtx, lv.gcmtx)
        self.gw_inv = np.linalg.inv(self.gw_mat)
        K = lv.kmax
        self.vd_inv = {}
        for name, nu in self.vcoef.items():
            self.vd_inv[name] = (None if nu is None else
                                 np.linalg.inv(np.eye(K) - dt * nu[:, None] * self.vlap))
        self._ops_dt = dt

    def implicit_step(self, dt, prev, tend):
        """Integrator.step, integrator.py:264-315."""
        self.prepare(dt)
        d, lv = self.damp, self.lv
        wt_vor, wt_div, wt_t, wt_pi, wt_q = tend
        ft = 1.0 + 2.0 * dt * d.ktt
        fd_hat = 1.0 + dt * d.kd
        wdx = prev["t"] * (1.0 + dt * d.ktt) + dt * wt_t
        wdphiy = lv.hydrostatic(wdx) + ft * ((prev["pi"] + dt * wt_pi)[..., None] * lv.gg)
        lap = self.tr.lap[:, None]
        rhs = prev["div"] * fd_hat * ft + dt * (wt_div * ft - lap * wdphiy)
        dbar = np.einsum("nij,...nj->...ni", self.gw_inv, rhs)
        wt_t = wt_t - np.einsum("kl,...l->...k", lv.tmtx, dbar)
        wt_pi = wt_pi - (dbar * lv.dsig).sum(axis=-1)
        new = {"vor": (prev["vor"] + 2.0 * dt * wt_vor) / (1.0 + 2.0 * dt * d.kv),
               "div": 2.0 * dbar - prev["div"],
               "t": (prev["t"] + 2.0 * dt * wt_t) / ft,
               "q": (prev["q"] + 2.0 * dt * wt_q) / (1.0 + 2.0 * dt * d.kq),
               "pi": prev["pi"] + 2.0 * dt * wt_pi}
        for name in ("vor", "div", "t", "q"):
            inv = self.vd_inv[name]
            if inv is None:
                continue
            out = np.einsum("ij,...j->...i", inv, new[name])
            if name in ("vor", "div"):        # integrator.py:236-239
                out[..., 0, :] = new[name][..., 0, :]
                out[..., 1, :] = new[name][..., 1, :]
            new[name] = out
        return new

    def step_dt(self, istep):
        c = self.cfg
        if istep > c.inistp:
            return c.delt, False
        return c.delt / 2.0 ** (c.inistp - istep + 1), True

    def step(self, frc_t=None, frc_vor=None, frc_div=None, frc_ps=None):
        """One call of the model.py:213-255 loop body."""
        self.istep += 1
        dt, start = self.step_dt(self.istep)
        tend = tendencies(self.tr, self.lv, self.bt, self.ga, frc_t=frc_t,
                          frc_vor=frc_vor, frc_div=frc_div, frc_ps=frc_ps,
                          strictly_linear=self.cfg.strictly_linear)
        prev = self.gb.to_spectral(self.tr)
        new_spec = self.implicit_step(dt, prev, tend)
        gc = GridState.from_spectral(self.tr, self.ga.ps_bar, new_spec)
        self.gb = self.ga.copy() if start else self.gb.filtered(self.ga, gc, self.cfg.robert)
        self.ga = gc
        if not self.ga.isfinite():
            raise FloatingPointError(f"model blew up at step {self.istep}")
        if not start:
            self.time += dt
            self.advanced += 1
        return new_spec

    def run(self, nsteps=None, frc_t=None, frc_vor=None, frc_div=None, frc_ps=None):
        """Advance `nsteps` advancing steps (default cfg.ndays), start-up included."""
        if nsteps is None:
            nsteps = int(round(self.cfg.ndays * self.cfg.steps_per_day))
        target = self.advanced + nsteps
        while self.advanced < target:
            self.step(frc_t=frc_t, frc_vor=frc_vor, frc_div=frc_div, frc_ps=frc_ps)
        return self
