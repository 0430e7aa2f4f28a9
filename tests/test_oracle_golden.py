"""Pin the CPU oracle against vectors produced by the reference itself.

The fixtures under tests/golden/ were generated by running the reference
package (tests/golden/make_golden.py).  Every quantity the GPU path is later
compared against is first checked here, so a parity failure on the GPU can
only mean a kernel bug, never an oracle bug.
"""

import json
import os
import types

import numpy as np
import pytest

from conftest import GOLDEN, golden, pack, relerr, unpack
from oracle import lbm_oracle as orc
from lbm_isca_gb300 import configs


def _t21():
    return orc.SphericalTransform(nlon=64, nlat=32, nmax=21)


def test_gauss_nodes_and_tables():
    g = golden("tables.npz")
    tr = _t21()
    assert relerr(tr.mu, g["t21_mu"]) < 1e-15
    assert relerr(tr.gw, g["t21_gw"]) < 1e-14
    assert relerr(tr.P, g["t21_P"]) < 1e-13
    assert relerr(tr.H, g["t21_H"]) < 1e-13
    t42 = orc.SphericalTransform()
    rows = list(g["t42_rows"])
    assert relerr(t42.P[rows], g["t42_P"]) < 1e-13
    assert relerr(t42.H[rows], g["t42_H"]) < 1e-13
    assert relerr(t42.gw, g["t42_gw"]) < 1e-14


@pytest.mark.parametrize("tag", ["t21", "t42"])
def test_transforms(tag):
    g = golden("transforms.npz")
    tr = _t21() if tag == "t21" else orc.SphericalTransform()
    M = tr.nmax + 1
    xi = unpack(g[f"{tag}_xi"], M)
    chi = unpack(g[f"{tag}_chi"], M)
    assert relerr(tr.wave_to_grid(xi), g[f"{tag}_w2g"]) < 1e-13
    assert relerr(pack(tr.grid_to_wave(g[f"{tag}_g1"]), M), g[f"{tag}_g2w"]) < 1e-13
    gx, gy = tr.hgrad(xi)
    assert relerr(gx, g[f"{tag}_gx"]) < 1e-13
    assert relerr(gy, g[f"{tag}_gy"]) < 1e-13
    vor, div = tr.uv_to_vordiv(g[f"{tag}_g1"], g[f"{tag}_g2"])
    assert relerr(pack(vor, M), g[f"{tag}_vor"]) < 1e-13
    assert relerr(pack(div, M), g[f"{tag}_div"]) < 1e-13
    u, v = tr.psichi_to_uv(xi * 1e6, chi * 1e6)
    assert relerr(u, g[f"{tag}_u"]) < 1e-13
    assert relerr(v, g[f"{tag}_v"]) < 1e-13


@pytest.mark.parametrize("tag", ["l20", "eq20"])
def test_vertical_operators(tag):
    g = golden("vertical.npz")
    sigm = orc.SIGMA_HALF_L20 if tag == "l20" else configs.equal_sigma_half_levels(20)
    lv = orc.SigmaLevels(sigm)
    lv.set_reference_temperature(200.0 + 3.0 * np.arange(lv.kmax))
    for name in ("sig", "dsig", "alpha", "dlog2", "dlog3", "cpg", "w3", "wP",
                 "dsigm", "ww", "tbar", "gg", "tmtx", "whmtx", "gcmtx"):
        assert relerr(getattr(lv, name), g[f"{tag}_{name}"]) < 1e-13, name


def _jet_basic(tr, lv):
    """The reference's synthetic baroclinic jet (analysis/tl_verification.py:67-77)."""
    nlat, nlon, k = tr.nlat, tr.nlon, lv.kmax
    lat = np.arcsin(tr.mu)[:, None, None]
    sig = lv.sig[None, None, :]
    jet = 30.0 * np.exp(-((lat - np.deg2rad(40)) / np.deg2rad(15)) ** 2)
    u = (jet * (sig ** 0.5)) * np.ones((nlat, nlon, k))
    t = (250.0 - 40.0 * np.sin(lat) ** 2 + 5.0 * sig) * np.ones((nlat, nlon, k))
    q = 1e-3 * np.exp(-((lat) / np.deg2rad(30)) ** 2) * np.ones((nlat, nlon, k))
    return types.SimpleNamespace(u=u, v=np.zeros((nlat, nlon, k)), t=t, q=q,
                                 ps=1.0e5 * np.ones((nlat, nlon)))


def test_operators_and_basic_terms():
    g = golden("operators_t21.npz")
    tr = _t21()
    sigm = configs.equal_sigma_half_levels(20)
    lv = orc.SigmaLevels(sigm)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    cfg = orc.RunConfig(**configs.plain_damping(20))
    m = orc.OracleModel(tr, lv, bs, cfg)
    m.prepare(cfg.delt)
    for name in ("kv", "kd", "ktt", "kq"):
        assert relerr(getattr(m.damp, name), g[name]) < 1e-14, name
    assert relerr(lv.tbar, g["tbar"]) < 1e-14
    assert relerr(m.gw_mat, g["semi_m"]) < 1e-14
    assert relerr(m.gw_inv, g["semi_minv"]) < 1e-12
    # default configuration on the reference L20 levels, jet basic state
    lvd = orc.SigmaLevels()
    md = orc.OracleModel(tr, lvd, _jet_basic(tr, lvd), orc.RunConfig())
    md.prepare(600.0)
    sub = (slice(None, None, 3), slice(None, None, 5))
    assert relerr(lvd.tbar, g["jet_tbar"]) < 1e-14
    for name in ("vor_g", "div", "pix", "piy", "sdot", "x5", "ssum"):
        assert relerr(getattr(md.bt, name)[sub], g[f"jet_{name}"]) < 1e-11, name
    for name in ("kv", "kd", "ktt", "kq"):
        assert relerr(getattr(md.damp, name), g[f"dflt_{name}"]) < 1e-14, name
    assert relerr(md.gw_inv, g["dflt_semi_minv"]) < 1e-12
    assert relerr(md.vd_inv["vor"], g["dflt_vd_vor"]) < 1e-12
    assert relerr(md.vd_inv["t"], g["dflt_vd_t"]) < 1e-12


def analytic_perturbation(tr, sig, scale=1.0):
    """Same analytic fields as tests/golden/make_golden.py."""
    la = np.arcsin(tr.mu)[:, None, None]
    lo = tr.lon[None, :, None]
    s = np.asarray(sig)[None, None, :]
    c = np.cos(la)
    u = scale * (2.0 * c ** 2 * np.sin(2 * lo) * (1 + s) + 0.5 * np.sin(la) * c * s)
    v = scale * (1.5 * c ** 3 * np.cos(3 * lo + 0.3) * (1.2 - s))
    t = scale * (1.0 * c ** 2 * np.cos(lo - 0.5) * np.sin(np.pi * s) + 0.3 * np.sin(2 * la))
    q = scale * 1e-3 * (c ** 4 * np.sin(lo + 1.0) * s)
    ps = scale * 2.0 * (c[..., 0] ** 2 * np.cos(2 * lo[..., 0] + 0.7))
    return u, v, t, q, ps


def test_tendencies():
    g = golden("tendencies_t21.npz")
    tr = _t21()
    lv = orc.SigmaLevels()
    bs = _jet_basic(tr, lv)
    bt = orc.BasicTerms(tr, lv, bs)
    u, v, t, q, ps = analytic_perturbation(tr, lv.sig)
    st = orc.GridState(bs.ps, u, v, t, q, ps)
    M = tr.nmax + 1
    diag = {}
    wt = orc.tendencies(tr, lv, bt, st, diag=diag)
    for name, x in zip(("vor", "div", "t", "pi", "q"), wt):
        assert relerr(pack(x, M), g[name]) < 1e-11, name
    assert relerr(diag["omega"][::4, ::4], g["omega"]) < 1e-11
    wl = orc.tendencies(tr, lv, bt, st, strictly_linear=True)
    assert relerr(pack(wl[1], M), g["div_lin"]) < 1e-11
    nlat, nlon = tr.nlat, tr.nlon
    lat = np.degrees(np.arcsin(tr.mu))
    lon = np.degrees(tr.lon)
    frc_t = 1e-5 * np.cos(np.radians(lat))[:, None, None] * np.ones((nlat, nlon, 20))
    frc_vor = 1e-11 * np.sin(np.radians(lon))[None, :, None] * np.ones((nlat, nlon, 20))
    frc_div = 2e-11 * np.cos(np.radians(lon))[None, :, None] * np.ones((nlat, nlon, 20))
    frc_ps = 1e-8 * np.cos(np.radians(lat))[:, None] * np.ones((nlat, nlon))
    wf = orc.tendencies(tr, lv, bt, st, frc_t=frc_t, frc_vor=frc_vor,
                        frc_div=frc_div, frc_ps=frc_ps)
    for name, x in zip(("vor", "div", "t", "pi", "q"), wf):
        assert relerr(pack(x, M), g[f"{name}_frc"]) < 1e-11, name


def _check_state(g, prefix, tr, st, lvl, tol):
    M = tr.nmax + 1
    spec = st.to_spectral(tr)
    for name in ("vor", "div", "t", "pi", "q"):
        ref = g[f"{prefix}_{lvl}_{name}"]
        got = pack(spec[name], M)
        if np.abs(ref).max() == 0.0:
            assert np.abs(got).max() < 1e-30, name
        else:
            assert relerr(got, ref) < tol, (prefix, lvl, name, relerr(got, ref))
    assert relerr(st.ps, g[f"{prefix}_{lvl}_ps"]) < tol


def test_run_plain_configuration():
    g = golden("runs_t21.npz")
    tr = _t21()
    sigm = configs.equal_sigma_half_levels(20)
    lv = orc.SigmaLevels(sigm)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    m = orc.OracleModel(tr, lv, bs, orc.RunConfig(**configs.plain_damping(20)))
    m.run(40, frc_t=configs.elliptic_heating(64, 32, sigm))
    assert m.istep == 42
    _check_state(g, "plain", tr, m.ga, "a", 1e-10)
    _check_state(g, "plain", tr, m.gb, "b", 1e-10)


def test_run_default_configuration():
    g = golden("runs_t21.npz")
    tr = _t21()
    lv = orc.SigmaLevels()
    bs = _jet_basic(tr, lv)
    m = orc.OracleModel(tr, lv, bs, orc.RunConfig())
    ub, vb, tb, qb, psb = analytic_perturbation(tr, lv.sig, 0.1)
    ub, vb = tr.vordiv_to_uv(*tr.uv_to_vordiv(ub, vb))
    m.set_initial_perturbation(u=ub, v=vb, t=tr.truncate(tb), q=tr.truncate(qb))
    heat = configs.elliptic_heating(64, 32, orc.SIGMA_HALF_L20, lon0=200.0, lat0=5.0)
    m.run(24, frc_t=heat)
    _check_state(g, "dflt", tr, m.ga, "a", 1e-10)
    _check_state(g, "dflt", tr, m.gb, "b", 1e-10)


def test_run_ensemble():
    g = golden("runs_t21.npz")
    tr = _t21()
    sigm = configs.equal_sigma_half_levels(20)
    lv = orc.SigmaLevels(sigm)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    heats, _ = configs.ensemble_heating(64, 32, sigm, 2, seed=1)
    m = orc.OracleModel(tr, lv, bs, orc.RunConfig(**configs.plain_damping(20)), nmem=2)
    m.run(12, frc_t=heats)
    _check_state(g, "ens", m.tr, m.ga, "a", 1e-10)


def gill_scales(u_eq, lon, lon0=180.0, radius=6.371e6):
    """Peak and e-folding analysis of analysis/gill_isca.py:59-90."""
    dlon = (lon - lon0 + 180.0) % 360.0 - 180.0
    order = np.argsort(dlon)
    dlon, u = dlon[order], u_eq[order]
    dist = np.radians(dlon) * radius / 1000.0
    east, west = dlon > 0, dlon < 0
    iE = np.nanargmax(np.abs(np.where(east, u, np.nan)))
    iW = np.nanargmax(np.abs(np.where(west, u, np.nan)))

    def efold(d, amp, lo, hi):
        sel = (d >= lo) & (d <= hi) & (amp > 0)
        slope = np.polyfit(d[sel], np.log(amp[sel]), 1)[0]
        return -1.0 / slope

    LK = efold(dist, np.where(east, np.abs(u), 0.0), dist[iE],
               np.radians(150) * radius / 1e3)
    LR = efold(-dist, np.where(west, np.abs(u), 0.0), -dist[iW],
               np.radians(85) * radius / 1e3)
    return dict(kelvin_peak_lon_offset_deg=dlon[iE], kelvin_peak_u_ms=u[iE],
                rossby_peak_lon_offset_deg=dlon[iW], rossby_peak_u_ms=u[iW],
                L_K_kelvin_efold_km=LK, L_R_rossby_efold_km=LR)


def gill_forcing(tr, lv, lon0=180.0, amp=1.0):
    """analysis/gill_isca.py:38-47: Gaussian equatorial heating, K/s."""
    lat = np.degrees(np.arcsin(tr.mu))
    lon = np.degrees(tr.lon)
    dl = (lon[None, :] - lon0 + 180.0) % 360.0 - 180.0
    hxy = np.exp(-(dl / 20.0) ** 2 - (lat[:, None] / 10.0) ** 2)
    vz = np.sin(np.pi * (1.0 - lv.sig)) * (lv.sig > 0.1)
    return hxy[:, :, None] * vz[None, None, :] * (amp / 86400.0)


def resting_state(tr, lv, t0=250.0):
    shape = (tr.nlat, tr.nlon, lv.kmax)
    return types.SimpleNamespace(u=np.zeros(shape), v=np.zeros(shape),
                                 t=np.full(shape, t0), q=np.zeros(shape),
                                 ps=np.full((tr.nlat, tr.nlon), 1000.0))


@pytest.mark.slow
def test_gill_day6_matches_reference_record():
    """6-day T42L20 Gill run reproduces the reference's recorded numbers."""
    with open(os.path.join(GOLDEN, "gill_record.json")) as fh:
        rec = json.load(fh)["cpu"]
    tr = orc.SphericalTransform()
    lv = orc.SigmaLevels()
    m = orc.OracleModel(tr, lv, resting_state(tr, lv), orc.RunConfig(ndays=6.0))
    m.run(frc_t=gill_forcing(tr, lv))
    assert m.advanced == 432 and m.istep == 434
    klo = int(np.argmin(np.abs(lv.sig - 0.85)))
    eq = int(np.argmin(np.abs(np.degrees(np.arcsin(tr.mu)))))
    got = gill_scales(m.ga.u[eq, :, klo], np.degrees(tr.lon))
    for key, val in got.items():
        assert abs(val - rec[key]) <= 1e-9 * max(1.0, abs(rec[key])), (key, val, rec[key])
