"""History records (GrADS), basic-state preprocessing and regridding against
fixtures produced by the reference itself (tests/golden/make_golden_io.py).

CPU tests: the .ctl descriptor, the pressure-level file reader, grid
detection.  GPU tests (the numerics run in the lbm_gb300 kernels): the day's
GrADS records byte for byte, z2ps / spline / p2s / zonal filter at 1e-12,
the whole basic-state pipeline and the regridding at 1e-10 (the transforms'
Gauss weights differ from numpy's by ~1e-13), a T21 <-> T42 round trip, and
history written by a fused run through ``LBM.run``."""

import os
import sys
import types

import numpy as np
import pytest

from conftest import GOLDEN, golden, relerr

sys.path.insert(0, GOLDEN)
import bs_inputs  # noqa: E402


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _grads_grid():
    sp = types.SimpleNamespace(nlon=16, nlat=8, lat_deg=bs_inputs.lat_deg(8))
    vg = types.SimpleNamespace(kmax=3, sig=np.array([0.95, 0.5, 0.1]))
    return sp, vg


def _grads_days(g):
    names = ("psi", "chi", "u", "v", "w", "t", "z", "p")
    return [{k: g[f"d{i}_{k}"] for k in names} for i in range(2)]


# ---------------------------------------------------------------- CPU tests
def test_grads_ctl_matches_reference(tmp_path):
    from lbm_isca_gb300.output import GradsWriter
    g = golden("grads.npz")
    sp, vg = _grads_grid()
    w = GradsWriter(str(tmp_path / "out.grd"), sp, vg, title="golden")
    w.ntime = 2
    assert w.ctl_text() == str(g["ctl"])
    w.fh.close()


def test_read_pressure_levels_matches_reference(tmp_path):
    from lbm_isca_gb300.basicstate import read_pressure_levels
    from lbm_isca_gb300.regrid import detect_grid
    b = golden("basicstate.npz")
    path = tmp_path / "bs.bin"
    b["rd_file"].tofile(path)
    assert detect_grid(str(path)) == (16, 8)
    r = read_pressure_levels(str(path), kmo=3, navg=3, nlon=16, nlat=8, nlev=3)
    for k in ("z", "q", "t", "u", "v"):
        np.testing.assert_array_equal(r[k], b[f"rd_{k}"])


def test_read_pressure_levels_rejects_bad_files(tmp_path):
    from lbm_isca_gb300.basicstate import read_pressure_levels
    b = golden("basicstate.npz")
    path = tmp_path / "bs.bin"
    b["rd_file"][:-4].tofile(path)
    with pytest.raises(ValueError):
        read_pressure_levels(str(path), nlon=16, nlat=8, nlev=3)
    b["rd_file"].tofile(path)
    with pytest.raises(ValueError):
        read_pressure_levels(str(path), nlon=8, nlat=16 * 2, nlev=3)    # wrong grid size
    with pytest.raises(ValueError):
        read_pressure_levels(str(path), kmo=5, navg=1, nlon=16, nlat=8, nlev=3)


# ---------------------------------------------------------------- GPU tests
@pytest.mark.gpu
def test_grads_records_match_reference_bytes(torch_cuda, tmp_path):
    from lbm_isca_gb300.output import GradsWriter
    torch = torch_cuda
    g = golden("grads.npz")
    sp, vg = _grads_grid()
    w = GradsWriter(str(tmp_path / "out.grd"), sp, vg, title="golden")
    for i, f in enumerate(_grads_days(g)):
        w.add(i + 1, {k: torch.as_tensor(v).cuda() for k, v in f.items()})
    w.close()
    got = np.fromfile(tmp_path / "out.grd", dtype=np.uint8)
    np.testing.assert_array_equal(got, g["grd"])
    assert open(tmp_path / "out.ctl").read() == str(g["ctl"])


@pytest.mark.gpu
def test_grads_host_input_and_shapes(torch_cuda, tmp_path):
    from lbm_isca_gb300.output import grads_records
    g = golden("grads.npz")
    day = _grads_days(g)[0]
    rec = grads_records(day, apply_z=False)
    n = 8 * 16
    assert len(rec) == (7 * 3 + 1) * (n + 2) * 4
    first = np.frombuffer(rec[:(n + 2) * 4], dtype=">f4")
    assert first[:1].view(">i4")[0] == 4 * n
    np.testing.assert_array_equal(first[1:-1], day["psi"][..., 0].astype(">f4").ravel())
    bad = dict(day, u=day["u"][..., :2])
    with pytest.raises(ValueError):
        grads_records(bad)


@pytest.mark.gpu
def test_column_kernels_match_reference(torch_cuda):
    from lbm_isca_gb300 import basicstate as bs
    b = golden("basicstate.npz")
    ps = bs.z2ps(b["z2ps_z"][None], b["z2ps_zs"][None])[0]
    assert relerr(ps, b["z2ps_ps"]) < 1e-12
    x = np.log(bs_inputs.PLEV17)
    assert relerr(bs.spline(x, b["sp_z"], b["sp_xi"]), b["sp_out"]) < 1e-12
    np.testing.assert_allclose(bs.spline(x, b["sp_z"], b["sp_xi"], omisb=True, omist=True),
                               b["sp_out_miss"], rtol=1e-12, atol=1e-9)
    assert relerr(bs.p2s(b["p2s_g"], b["p2s_ps"], b["p2s_sig"]), b["p2s_out"]) < 1e-12
    assert relerr(bs.zmsw(b["zm_in"], ozm=True), b["zm_ozm"]) < 1e-12
    assert relerr(bs.zmsw(b["zm_in"], osw=True), b["zm_osw"]) < 1e-12
    np.testing.assert_array_equal(bs.zmsw(b["zm_in"]), b["zm_in"])


@pytest.mark.gpu
def test_load_basic_state_matches_reference(torch_cuda, tmp_path):
    from lbm_isca_gb300 import Spectral, VerticalGrid
    from lbm_isca_gb300.basicstate import load_basic_state
    b = golden("basicstate.npz")
    path = str(tmp_path / "bs_t21.bin")
    bs_inputs.write_pressure_file(path, nlon=64, nlat=32, nlev=17, nmonth=3, seed=9)
    sp = Spectral(nlon=64, nlat=32, nmax=21)
    vg = VerticalGrid(sigm=bs_inputs.SIGM5)
    st = load_basic_state(path, sp, vg, kmo=1, navg=2)
    for k in ("u", "v", "t", "q"):
        a = getattr(st, k)
        assert a.shape == (32, 64, 5)
        assert relerr(a.reshape(-1, 5)[::7], b[f"lbs_{k}"]) < 1e-10, k
    assert relerr(st.ps.reshape(-1)[::7], b["lbs_ps"]) < 1e-10


@pytest.mark.gpu
def test_regrid_matches_reference(torch_cuda):
    from lbm_isca_gb300 import Spectral
    from lbm_isca_gb300 import regrid as rg
    r = golden("regrid.npz")
    sp21, sp10 = Spectral(nlon=64, nlat=32, nmax=21), Spectral(nlon=64, nlat=32, nmax=10)
    for tag, a, c in (("dn", sp21, sp10), ("up", sp10, sp21)):
        assert relerr(rg.regrid_scalar(a, c, r["s2"]).reshape(-1)[::4], r[f"{tag}_s2"]) < 1e-10
        s3 = rg.regrid_scalar(a, c, r["s3"])
        assert relerr(s3.reshape(-1, 2)[::4], r[f"{tag}_s3"]) < 1e-10
        u, v = rg.regrid_uv(a, c, r["u"], r["v"])
        assert relerr(u.reshape(-1)[::4], r[f"{tag}_u"]) < 1e-10
        assert relerr(v.reshape(-1)[::4], r[f"{tag}_v"]) < 1e-10


@pytest.mark.gpu
def test_regrid_t21_t42_round_trip(torch_cuda):
    """Up to the T42 grid and back recovers the T21-truncated field."""
    from lbm_isca_gb300 import Spectral
    from lbm_isca_gb300 import regrid as rg
    from lbm_isca_gb300.forcing import MJOForcing
    sp21, sp42 = Spectral(nlon=64, nlat=32, nmax=21), Spectral(nlon=128, nlat=64, nmax=42)
    s2, s3, u, v = bs_inputs.regrid_fields(sp21.lat_deg)
    base = np.asarray(sp21.truncate(s3).cpu())
    back = rg.regrid_scalar(sp42, sp21, rg.regrid_scalar(sp21, sp42, base))
    assert relerr(back, base) < 1e-11
    u0, v0 = (np.asarray(x.cpu()) for x in sp21.vordiv_to_uv(*sp21.uv_to_vordiv(u, v)))
    u1, v1 = rg.regrid_uv(sp42, sp21, *rg.regrid_uv(sp21, sp42, u0, v0))
    assert relerr(u1, u0) < 1e-11 and relerr(v1, v0) < 1e-11
    gtf = np.stack([s3, 2.0 * s3, -s3])                 # (day, lat, lon, lev)
    mjo = MJOForcing(gtf, nt=4, spinup=2)
    mjo.step()
    rg.regrid_mjo_forcing(mjo, sp21, sp42)
    assert mjo.gtf.shape == (3, 64, 128, 2) and mjo.counter == 0
    assert relerr(mjo.gtf[1], rg.regrid_scalar(sp21, sp42, 2.0 * s3)) < 1e-13


@pytest.mark.gpu
def test_fused_run_writes_grads_history(torch_cuda, tmp_path):
    """A fused run with a GradsWriter writes, per day, the reference's
    encoding of the fields a plain collecting writer receives."""
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid, configs
    from lbm_isca_gb300.constants import GRAV_GT2GR, RHO00
    from lbm_isca_gb300.output import GradsWriter

    class Collect:
        def __init__(self):
            self.days = []

        def add(self, day, fields):
            self.days.append({k: np.array(v) for k, v in fields.items()})

        def close(self):
            pass

    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    heat = configs.elliptic_heating(64, 32, sigm)
    steady = types.SimpleNamespace(vor=np.zeros_like(heat), div=np.zeros_like(heat),
                                   ps=np.zeros((32, 64)), t=heat)

    def run(writer):
        sp = Spectral(nlon=64, nlat=32, nmax=21)
        vg = VerticalGrid(sigm=sigm)
        cfg = Config(ndays=2.0, **configs.plain_damping(20))
        LBM(bs, sp, vg, cfg).run(steady_forcing=steady, writer=writer, verbose=False)

    col = Collect()
    run(col)
    sp, vg = Spectral(nlon=64, nlat=32, nmax=21), VerticalGrid(sigm=sigm)
    w = GradsWriter(str(tmp_path / "h.grd"), sp, vg)
    run(w)
    assert len(col.days) == 2 and w.ntime == 2
    got = np.fromfile(tmp_path / "h.grd", dtype=np.uint8)
    expect = []
    for f in col.days:
        f = dict(f)
        f["z"] = f["z"] + f["p"][..., None] * 1.0e2 / (RHO00 * GRAV_GT2GR)
        for name in ("psi", "chi", "u", "v", "w", "t", "z", "p"):
            a = f[name]
            for k in range(a.shape[-1] if a.ndim == 3 else 1):
                rec = (a[..., k] if a.ndim == 3 else a).astype(">f4").ravel()
                mark = np.array([rec.size * 4], dtype=">i4")
                expect += [mark.tobytes(), rec.tobytes(), mark.tobytes()]
    np.testing.assert_array_equal(got, np.frombuffer(b"".join(expect), dtype=np.uint8))
