"""GPU parity of the tendencies, implicit step and full time loop (general and
fused) against the reference's golden vectors and the CPU oracle."""

import json
import os
import types

import numpy as np
import pytest

from conftest import GOLDEN, golden, pack, relerr, unpack
from oracle import lbm_oracle as orc
from lbm_isca_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _np(x):
    return x.detach().cpu().numpy()


def _jet_basic(mu, sig, nlat, nlon):
    """analysis/tl_verification.py:67-77 synthetic baroclinic jet."""
    k = sig.size
    lat = np.arcsin(mu)[:, None, None]
    s = sig[None, None, :]
    jet = 30.0 * np.exp(-((lat - np.deg2rad(40)) / np.deg2rad(15)) ** 2)
    u = (jet * (s ** 0.5)) * np.ones((nlat, nlon, k))
    t = (250.0 - 40.0 * np.sin(lat) ** 2 + 5.0 * s) * np.ones((nlat, nlon, k))
    q = 1e-3 * np.exp(-(lat / np.deg2rad(30)) ** 2) * np.ones((nlat, nlon, k))
    return types.SimpleNamespace(u=u, v=np.zeros((nlat, nlon, k)), t=t, q=q,
                                 ps=1.0e5 * np.ones((nlat, nlon)))


def _perturbation(mu, lon, sig, scale=1.0):
    la = np.arcsin(mu)[:, None, None]
    lo = lon[None, :, None]
    s = sig[None, None, :]
    c = np.cos(la)
    u = scale * (2.0 * c ** 2 * np.sin(2 * lo) * (1 + s) + 0.5 * np.sin(la) * c * s)
    v = scale * (1.5 * c ** 3 * np.cos(3 * lo + 0.3) * (1.2 - s))
    t = scale * (1.0 * c ** 2 * np.cos(lo - 0.5) * np.sin(np.pi * s) + 0.3 * np.sin(2 * la))
    q = scale * 1e-3 * (c ** 4 * np.sin(lo + 1.0) * s)
    ps = scale * 2.0 * (c[..., 0] ** 2 * np.cos(2 * lo[..., 0] + 0.7))
    return u, v, t, q, ps


def _t21():
    from lbm_isca_gb300 import Spectral
    return Spectral(nlon=64, nlat=32, nmax=21, device="gb300")


def test_tendencies_vs_golden():
    from lbm_isca_gb300 import VerticalGrid, State
    from lbm_isca_gb300.dynamics import BasicStateTerms, Dynamics
    g = golden("tendencies_t21.npz")
    sp = _t21()
    vg = VerticalGrid(device="gb300")
    sig = vg.host("sig")
    bs = _jet_basic(sp.mu, sig, 32, 64)
    bst = BasicStateTerms(sp, vg, bs)
    u, v, t, q, ps = _perturbation(sp.mu, sp.lon, sig)
    st = State(bs.ps, u=u, v=v, t=t, q=q, ps=ps, device="gb300")
    M = 22
    dyn = Dynamics(sp, vg, bst)
    wt = dyn.tendencies(st)
    for name, x in zip(("vor", "div", "t", "q"), (wt[0], wt[1], wt[2], wt[4])):
        assert relerr(pack(_np(x), M), g[name]) < 1e-10, name
    # The reference forms gt_pi = -S[0] + sum(dsig div), two O(|div|) terms
    # cancelling to O(|v.grad pi|): here 1e-6 vs 1e-11, so its value carries
    # ~K eps |sum dsig div| of rounding; the kernel sums -dsig v.grad(pi)
    # directly.  Compare within the reference's own rounding floor.
    div_s = sp.uv_to_vordiv(st.u, st.v)[1]
    sdiv = (sp.wave_to_grid(div_s) * vg.dsig).sum(-1).abs().max().item()
    floor = 20 * 4 * 2.2e-16 * sdiv
    diff = np.abs(pack(_np(wt[3]), M) - g["pi"]).max()
    assert diff < max(1e-10 * np.abs(g["pi"]).max(), floor), (diff, floor)
    assert relerr(_np(dyn.diag["omega"])[::4, ::4], g["omega"]) < 1e-10
    wl = Dynamics(sp, vg, bst, strictly_linear=True).tendencies(st)
    assert relerr(pack(_np(wl[1]), M), g["div_lin"]) < 1e-10
    lat, lon = sp.lat_deg, sp.lon_deg
    frc_t = 1e-5 * np.cos(np.radians(lat))[:, None, None] * np.ones((32, 64, 20))
    frc_vor = 1e-11 * np.sin(np.radians(lon))[None, :, None] * np.ones((32, 64, 20))
    frc_div = 2e-11 * np.cos(np.radians(lon))[None, :, None] * np.ones((32, 64, 20))
    frc_ps = 1e-8 * np.cos(np.radians(lat))[:, None] * np.ones((32, 64))
    wf = dyn.tendencies(st, frc_t=frc_t, frc_vor=frc_vor, frc_div=frc_div, frc_ps=frc_ps)
    for name, x in zip(("vor", "div", "t", "pi", "q"), wf):
        assert relerr(pack(_np(x), M), g[f"{name}_frc"]) < 1e-10, name


def test_resting_state_gives_zero_tendency():
    """The reference's test_physics_isca.py:56-61: exactly zero."""
    from lbm_isca_gb300 import Spectral, VerticalGrid, LBM, Config
    sp = Spectral(device="gb300")
    vg = VerticalGrid(device="gb300")
    shape = (64, 128, 20)
    bs = types.SimpleNamespace(u=np.zeros(shape), v=np.zeros(shape),
                               t=np.full(shape, 250.0), q=np.zeros(shape),
                               ps=np.full((64, 128), 1000.0))
    m = LBM(bs, sp, vg, Config(ndays=0.1))
    for name, x in zip(("vor", "div", "t", "pi", "q"), m.dyn.tendencies(m.ga)):
        assert float(x.abs().max()) == 0.0, name


def test_semi_implicit_operators():
    from lbm_isca_gb300 import LBM, Config, VerticalGrid
    g = golden("operators_t21.npz")
    sp = _t21()
    sigm = configs.equal_sigma_half_levels(20)
    vg = VerticalGrid(sigm=sigm, device="gb300")
    bs = configs.solid_body_basic_state(64, 32, sigm)
    m = LBM(bs, sp, vg, Config(ndays=1.0, **configs.plain_damping(20)))
    m.semi.prepare(1200.0)
    for name in ("kv", "kd", "ktt", "kq"):
        assert relerr(_np(getattr(m.damping, name)), g[name]) < 1e-14
    assert relerr(_np(m.semi.m), g["semi_m"]) < 1e-13
    assert relerr(_np(m.semi.minv), g["semi_minv"]) < 1e-12
    assert m.semi.cond.max() < 100.0
    resid = np.einsum("nij,njk->nik", _np(m.semi.m), _np(m.semi.minv))
    assert np.abs(resid - np.eye(20)).max() < 1e-10


def test_implicit_step_vs_oracle():
    from lbm_isca_gb300 import LBM, Config, VerticalGrid
    sp = _t21()
    vg = VerticalGrid(device="gb300")
    tr = orc.SphericalTransform(64, 32, 21)
    lv = orc.SigmaLevels()
    bs = _jet_basic(sp.mu, vg.host("sig"), 32, 64)
    m = LBM(bs, sp, vg, Config())
    om = orc.OracleModel(tr, lv, bs, orc.RunConfig())
    rng = np.random.default_rng(4)
    M = 22
    mask = tr.mask

    def rnd(shape):
        x = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        x[~mask] = 0.0
        x[0] = x[0].real
        return x
    prev = {k: rnd((M, M, 20)) for k in ("vor", "div", "t", "q")}
    prev["pi"] = rnd((M, M)) * 1e-3
    tend = [rnd((M, M, 20)) * 1e-6 for _ in range(3)] + [rnd((M, M)) * 1e-9,
                                                          rnd((M, M, 20)) * 1e-9]
    for dt in (300.0, 1200.0):
        got = m.integ.step(dt, prev, tend)
        ref = om.implicit_step(dt, prev, tend)
        for k in ("vor", "div", "t", "pi", "q"):
            assert relerr(_np(got[k]), ref[k]) < 1e-12, (dt, k)


def _check(g, prefix, lvl, sp, st, tol):
    M = sp.nmax + 1
    spec = st.to_spectral(sp)
    for name in ("vor", "div", "t", "pi", "q"):
        ref = g[f"{prefix}_{lvl}_{name}"]
        got = pack(_np(spec[name]), M)
        if np.abs(ref).max() == 0.0:
            assert np.abs(got).max() < 1e-25, (prefix, lvl, name)
        else:
            e = relerr(got, ref)
            assert e < tol, (prefix, lvl, name, e)
    assert relerr(_np(st.ps), g[f"{prefix}_{lvl}_ps"]) < tol


def _plain_model(fused, precision="fp64"):
    from lbm_isca_gb300 import LBM, Config, VerticalGrid
    sp = _t21()
    sigm = configs.equal_sigma_half_levels(20)
    vg = VerticalGrid(sigm=sigm, device="gb300")
    bs = configs.solid_body_basic_state(64, 32, sigm)
    cfg = Config(ndays=40 / 72.0, fused=fused, precision=precision,
                 **configs.plain_damping(20))
    return LBM(bs, sp, vg, cfg), sigm


class _Steady:
    def __init__(self, t, nlat, nlon, K):
        self.t = t
        self.vor = np.zeros_like(t)
        self.div = np.zeros_like(t)
        self.ps = np.zeros((nlat, nlon))


@pytest.mark.parametrize("fused", [False, True])
def test_run_plain_configuration(fused):
    g = golden("runs_t21.npz")
    m, sigm = _plain_model(fused)
    heat = configs.elliptic_heating(64, 32, sigm)
    m.run(steady_forcing=_Steady(heat, 32, 64, 20), verbose=False)
    _check(g, "plain", "a", m.sp, m.ga, 1e-10)
    _check(g, "plain", "b", m.sp, m.gb, 1e-10)


def test_run_plain_configuration_fp32():
    g = golden("runs_t21.npz")
    m, sigm = _plain_model(True, "fp32")
    heat = configs.elliptic_heating(64, 32, sigm)
    m.run(steady_forcing=_Steady(heat, 32, 64, 20), verbose=False)
    _check(g, "plain", "a", m.sp, m.ga, 1e-5)


@pytest.mark.parametrize("fused", [False, True])
def test_run_default_configuration(fused):
    """Sponge, vertical diffusion, jet basic state, non-zero initial state."""
    from lbm_isca_gb300 import LBM, Config, VerticalGrid
    g = golden("runs_t21.npz")
    sp = _t21()
    vg = VerticalGrid(device="gb300")
    sig = vg.host("sig")
    bs = _jet_basic(sp.mu, sig, 32, 64)
    m = LBM(bs, sp, vg, Config(ndays=24 / 72.0, fused=fused))
    ub, vb, tb, qb, _ = _perturbation(sp.mu, sp.lon, sig, 0.1)
    tr = orc.SphericalTransform(64, 32, 21)
    ub, vb = tr.vordiv_to_uv(*tr.uv_to_vordiv(ub, vb))
    m.set_initial_perturbation(u=ub, v=vb, t=tr.truncate(tb), q=tr.truncate(qb))
    heat = configs.elliptic_heating(64, 32, orc.SIGMA_HALF_L20, lon0=200.0, lat0=5.0)
    m.run(steady_forcing=_Steady(heat, 32, 64, 20), verbose=False)
    _check(g, "dflt", "a", sp, m.ga, 1e-10)
    _check(g, "dflt", "b", sp, m.gb, 1e-10)


def test_run_ensemble():
    from lbm_isca_gb300 import Config
    from lbm_isca_gb300.ensemble import EnsembleForcing, make_ensemble_model
    g = golden("runs_t21.npz")
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    heats, _ = configs.ensemble_heating(64, 32, sigm, 2, seed=1)
    m, spb, vg = make_ensemble_model(bs, 2, Config(ndays=12 / 72.0,
                                                   **configs.plain_damping(20)),
                                     device="gb300", nlon=64, nlat=32, nmax=21, sigm=sigm)
    m.run(mjo_forcing=EnsembleForcing(heats, device="gb300"), verbose=False)
    _check(g, "ens", "a", spb, m.ga, 1e-10)


def test_gill_day6_matches_reference_record():
    """analysis/gill_isca.json: T42L20 Gill run, day 6 (432 + 2 steps)."""
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid
    from test_oracle_golden import gill_forcing, gill_scales, resting_state
    with open(os.path.join(GOLDEN, "gill_record.json")) as fh:
        rec = json.load(fh)["cpu"]
    sp = Spectral(device="gb300")
    vg = VerticalGrid(device="gb300")
    tr = orc.SphericalTransform()
    lv = orc.SigmaLevels()
    m = LBM(resting_state(tr, lv), sp, vg, Config(ndays=6.0))
    m.run(steady_forcing=_Steady(gill_forcing(tr, lv), 64, 128, 20), verbose=False)
    klo = int(np.argmin(np.abs(lv.sig - 0.85)))
    eq = int(np.argmin(np.abs(sp.lat_deg)))
    got = gill_scales(_np(m.ga.u)[eq, :, klo], sp.lon_deg)
    for key, val in got.items():
        assert abs(val - rec[key]) <= 1e-9 * max(1.0, abs(rec[key])), (key, val, rec[key])
    d = m.diagnostics()
    assert set(d) == {"psi", "chi", "u", "v", "w", "t", "z", "p"}


def test_fp32_ensemble_within_1e5_of_fp64_at_day10():
    """The FP32 stepper stays within 1e-5 relative L2 of the FP64 stepper (which
    equals the oracle to 1e-10) for every prognostic field after 10 days at
    T42L20: seeded elliptic heatings, solid-body basic state, plain damping."""
    import torch
    from lbm_isca_gb300 import Config
    from lbm_isca_gb300.ensemble import EnsembleForcing, make_ensemble_model
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(128, 64, sigm)
    heats, _ = configs.ensemble_heating(128, 64, sigm, 4, seed=1)
    out = {}
    for prec in ("fp64", "fp32"):
        m, _, _ = make_ensemble_model(
            bs, 4, Config(ndays=10.0, precision=prec, **configs.plain_damping(20)),
            device="gb300", nlon=128, nlat=64, nmax=42, sigm=sigm)
        m.run(mjo_forcing=EnsembleForcing(heats, device="gb300"), verbose=False)
        a, _ = m.stepper().spectral_state()
        out[prec] = {k: v.cpu() for k, v in a.items()}
    for k in ("vor", "div", "t", "pi"):
        r, f = out["fp64"][k], out["fp32"][k]
        e = float(torch.linalg.norm(f - r) / torch.linalg.norm(r))
        assert e <= 1e-5, (k, e)


class _Writer:
    """Collects the history records the model writes (output.py's protocol)."""

    def __init__(self):
        self.days = []
        self.closed = False

    def add(self, day, fields):
        self.days.append((day, {k: np.array(v) for k, v in fields.items()}))

    def close(self):
        self.closed = True


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 2e-5)])
def test_fused_history_matches_general_loop(precision, tol):
    """Daily trapezoid-mean history (model.py:257-277) accumulated on the
    device by the fused stepper equals the general loop's per-step average."""
    from lbm_isca_gb300 import LBM, Config, VerticalGrid
    sp = _t21()
    sigm = configs.equal_sigma_half_levels(20)
    vg = VerticalGrid(sigm=sigm, device="gb300")
    bs = configs.solid_body_basic_state(64, 32, sigm)
    heat = configs.elliptic_heating(64, 32, sigm)
    out = {}
    for fused, prec in ((False, "fp64"), (True, precision)):
        cfg = Config(ndays=2.0, fused=fused, precision=prec, **configs.plain_damping(20))
        w = _Writer()
        LBM(bs, sp, vg, cfg).run(steady_forcing=_Steady(heat, 32, 64, 20), writer=w,
                                 verbose=False)
        assert w.closed and [d for d, _ in w.days] == [1, 2]
        out[fused] = w.days
    for (_, ref), (_, got) in zip(out[False], out[True]):
        assert set(ref) == {"psi", "chi", "u", "v", "w", "t", "z", "p"}
        for k in ref:
            e = np.linalg.norm(got[k] - ref[k]) / np.linalg.norm(ref[k])
            assert e < tol, (k, e)


def _t85l40_model(fused, precision, ndays):
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid
    sp = Spectral(nlon=256, nlat=128, nmax=85, device="gb300")
    sigm = configs.equal_sigma_half_levels(40)
    vg = VerticalGrid(sigm=sigm, device="gb300")
    bs = configs.solid_body_basic_state(256, 128, sigm)
    cfg = Config(ndays=ndays, fused=fused, precision=precision, **configs.plain_damping(40))
    return LBM(bs, sp, vg, cfg), sigm


def test_t85l40_fused_matches_general_loop():
    """The largest configuration (T85L40, 256x128 grid): the fused FP64
    stepper against the reference step sequence (general loop) over 6 steps,
    and the FP32 stepper against FP64 over 4 model hours."""
    ndays = 6 / 72.0
    res = {}
    for fused, prec in ((False, "fp64"), (True, "fp64")):
        m, sigm = _t85l40_model(fused, prec, ndays)
        heat = configs.elliptic_heating(256, 128, sigm)
        m.run(steady_forcing=_Steady(heat, 128, 256, 40), verbose=False)
        res[(fused, prec)] = m.ga
    for k in ("u", "v", "t", "ps"):
        r, g = _np(getattr(res[(False, "fp64")], k)), _np(getattr(res[(True, "fp64")], k))
        assert relerr(g, r) < 1e-10, k
    m, sigm = _t85l40_model(True, "fp32", ndays)
    heat = configs.elliptic_heating(256, 128, sigm)
    m.run(steady_forcing=_Steady(heat, 128, 256, 40), verbose=False)
    for k in ("u", "v", "t", "ps"):
        r, g = _np(getattr(res[(True, "fp64")], k)), _np(getattr(m.ga, k))
        assert relerr(g, r) < 1e-5, k


def test_steady_forcing_all_channels_fused_matches_general():
    """Steady forcing through every channel the reference accepts (vor, div,
    T on levels and ps, dynamics.py:189-190, 248-251; forcing.py:71-96): the
    fused stepper (spectral forcing) against the general loop (grid forcing)
    over one day at T21L20."""
    from lbm_isca_gb300 import LBM, Config, VerticalGrid
    sp = _t21()
    sigm = configs.equal_sigma_half_levels(20)
    vg = VerticalGrid(sigm=sigm, device="gb300")
    bs = configs.solid_body_basic_state(64, 32, sigm)
    heat = configs.elliptic_heating(64, 32, sigm)
    lat = np.arcsin(sp.mu)[:, None]
    lon = sp.lon[None, :]
    shape2 = np.cos(lat) ** 2 * np.sin(2 * lon)
    frc = _Steady(heat, 32, 64, 20)
    frc.vor = 1e-11 * shape2[..., None] * np.ones(20)
    frc.div = 5e-12 * np.cos(lat)[..., None] * np.cos(lon)[..., None] * np.ones(20)
    frc.ps = 1e-5 * shape2
    out = {}
    for fused in (False, True):
        m = LBM(bs, sp, vg, Config(ndays=1.0, fused=fused, **configs.plain_damping(20)))
        m.run(steady_forcing=frc, verbose=False)
        out[fused] = m.ga
    for k in ("u", "v", "t", "ps"):
        assert relerr(_np(getattr(out[True], k)), _np(getattr(out[False], k))) < 1e-10, k


def test_mjo_forcing_spectral_interpolation_matches_general_loop():
    """Daily-record MJO forcing: the fused stepper's on-device spectral
    interpolation against the general loop's per-step grid field."""
    from lbm_isca_gb300 import LBM, Config, VerticalGrid
    from lbm_isca_gb300.forcing import MJOForcing
    sp = _t21()
    sigm = configs.equal_sigma_half_levels(20)
    vg = VerticalGrid(sigm=sigm, device="gb300")
    bs = configs.solid_body_basic_state(64, 32, sigm)
    days = np.stack([configs.elliptic_heating(64, 32, sigm, lon0=lon, lat0=5.0)
                     for lon in (90.0, 120.0, 150.0)])
    out = {}
    for fused in (False, True):
        f = MJOForcing(days, nt=72, spinup=20)
        m = LBM(bs, sp, vg, Config(ndays=2.0, fused=fused, **configs.plain_damping(20)))
        m.run(mjo_forcing=f, verbose=False)
        out[fused] = m.ga
        assert f.counter == 2 * 72 + 2
    for k in ("u", "v", "t", "ps"):
        assert relerr(_np(getattr(out[True], k)), _np(getattr(out[False], k))) < 1e-10, k


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_blowup_names_the_member_and_leaves_the_others_untouched(precision):
    """A NaN put into one member's heating on the host makes the run raise
    FloatingPointError (model.py:245-247) naming that member and a window of
    steps; every other member's state is bitwise that of a clean run."""
    import torch
    from lbm_isca_gb300 import Config
    from lbm_isca_gb300.ensemble import EnsembleForcing, make_ensemble_model
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    heats, _ = configs.ensemble_heating(64, 32, sigm, 4, seed=3)
    bad = heats.copy()
    bad[2, 10, 20, 5] = np.nan
    states = {}
    for name, h in (("clean", heats), ("nan", bad)):
        m, _, _ = make_ensemble_model(
            bs, 4, Config(ndays=0.5, precision=precision, **configs.plain_damping(20)),
            device="gb300", nlon=64, nlat=32, nmax=21, sigm=sigm)
        if name == "nan":
            with pytest.raises(FloatingPointError, match=r"member 2\b") as ex:
                m.run(mjo_forcing=EnsembleForcing(h, device="gb300"), verbose=False)
            assert "between 1 and" in str(ex.value)
        else:
            m.run(mjo_forcing=EnsembleForcing(h, device="gb300"), verbose=False)
        stp = m.stepper()
        torch.cuda.synchronize()
        # the spectral levels (the clean run's unload updates only the grid ps')
        states[name] = (stp.sa3.clone(), stp.sb3.clone(), stp.sas.clone())
        assert stp.bad_members() == ([2] if name == "nan" else [])
    for c, n in zip(states["clean"], states["nan"]):
        assert not torch.isfinite(n[2]).all()
        for e in (0, 1, 3):
            assert torch.equal(c[e], n[e]), e
