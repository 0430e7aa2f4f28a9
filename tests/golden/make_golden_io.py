#!/usr/bin/env python3
"""Golden fixtures for the formats and setup steps around the hot path,
generated by running the reference package itself:

* ``grads.npz``: two days of seeded history fields through the reference's
  ``GradsWriter`` (the .grd bytes and the .ctl text);
* ``basicstate.npz``: ``z2ps``, ``spline`` (with and without missing ends),
  ``p2s``, ``zmsw``, ``read_pressure_levels`` on a synthetic file (its bytes
  are stored) and ``load_basic_state`` end to end on a T21 grid (every 7th
  grid column of the result);
* ``regrid.npz``: ``regrid_scalar`` and ``regrid_uv`` between T21 and T10 on
  the 64 x 32 grid (every 4th point of the result).

Usage (where the reference checkout is available):

    python tests/golden/make_golden_io.py <path of the reference checkout>

Inputs come from ``bs_inputs.py`` next to this script (seeded, shared with
the tests).
"""

import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import bs_inputs  # noqa: E402


def grads(ref_output):
    sp = types.SimpleNamespace(nlon=16, nlat=8, lat_deg=bs_inputs.lat_deg(8))
    vg = types.SimpleNamespace(kmax=3, sig=np.array([0.95, 0.5, 0.1]))
    days = bs_inputs.history_days(nlat=8, nlon=16, kmax=3, ndays=2)
    with tempfile.TemporaryDirectory() as d:
        w = ref_output.GradsWriter(os.path.join(d, "out.grd"), sp, vg, title="golden")
        for i, f in enumerate(days):
            w.add(i + 1, {k: v.copy() for k, v in f.items()})
        w.close()
        grd = np.fromfile(os.path.join(d, "out.grd"), dtype=np.uint8)
        ctl = open(os.path.join(d, "out.ctl")).read()
    out = {"grd": grd, "ctl": np.array(ctl)}
    for i, f in enumerate(days):
        for k, v in f.items():
            out[f"d{i}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "grads.npz"), **out)


def basic_state(ref, bs):
    out = {}
    z, zs = bs_inputs.heights(ncol=48)
    out["z2ps_z"], out["z2ps_zs"] = z, zs
    out["z2ps_ps"] = bs.z2ps(z[None], zs[None])[0]
    x = np.log(bs_inputs.PLEV17)
    zc, xi = bs_inputs.spline_case(ncol=40)
    out["sp_z"], out["sp_xi"] = zc, xi
    out["sp_out"] = bs.spline(x, zc, xi)
    out["sp_out_miss"] = bs.spline(x, zc, xi, omisb=True, omist=True)
    g, ps, sig = bs_inputs.p2s_case()
    out["p2s_g"], out["p2s_ps"], out["p2s_sig"] = g, ps, sig
    out["p2s_out"] = bs.p2s(g, ps, sig)
    f = bs_inputs.zonal_case()
    out["zm_in"] = f
    out["zm_ozm"] = bs.zmsw(f, ozm=True)
    out["zm_osw"] = bs.zmsw(f, osw=True)
    with tempfile.TemporaryDirectory() as d:
        # small file: 16 x 8 grid, 3 pressure levels, 4 months
        path = os.path.join(d, "bs_small.bin")
        bs_inputs.write_pressure_file(path, nlon=16, nlat=8, nlev=3, nmonth=4, seed=5, undef=True)
        out["rd_file"] = np.fromfile(path, dtype=np.uint8)
        r = bs.read_pressure_levels(path, kmo=3, navg=3, nlon=16, nlat=8, nlev=3)
        for k, v in r.items():
            out[f"rd_{k}"] = v
        # end to end on the T21 grid, 17 levels, 3 months
        path = os.path.join(d, "bs_t21.bin")
        bs_inputs.write_pressure_file(path, nlon=64, nlat=32, nlev=17, nmonth=3, seed=9)
        sp = ref.Spectral(nlon=64, nlat=32, nmax=21, device="cpu")
        vg = ref.VerticalGrid(sigm=bs_inputs.SIGM5, device="cpu")
        b = bs.load_basic_state(path, sp, vg, kmo=1, navg=2)
        for k in ("u", "v", "t", "q"):
            out[f"lbs_{k}"] = getattr(b, k).reshape(-1, getattr(b, k).shape[-1])[::7]
        out["lbs_ps"] = b.ps.reshape(-1)[::7]
    np.savez_compressed(os.path.join(HERE, "basicstate.npz"), **out)


def regrid(ref, rg):
    sp21 = ref.Spectral(nlon=64, nlat=32, nmax=21, device="cpu")
    sp10 = ref.Spectral(nlon=64, nlat=32, nmax=10, device="cpu")
    s2, s3, u, v = bs_inputs.regrid_fields(sp21.lat_deg)
    out = {"s2": s2, "s3": s3, "u": u, "v": v}
    for tag, a, b in (("dn", sp21, sp10), ("up", sp10, sp21)):
        out[f"{tag}_s2"] = rg.regrid_scalar(a, b, s2).reshape(-1)[::4]
        out[f"{tag}_s3"] = rg.regrid_scalar(a, b, s3).reshape(-1, s3.shape[-1])[::4]
        uu, vv = rg.regrid_uv(a, b, u, v)
        out[f"{tag}_u"], out[f"{tag}_v"] = uu.reshape(-1)[::4], vv.reshape(-1)[::4]
    np.savez_compressed(os.path.join(HERE, "regrid.npz"), **out)


def main(refdir):
    sys.path.insert(0, refdir)
    import pylbm_isca as ref
    from pylbm_isca import basicstate as bs
    from pylbm_isca import output as ref_output
    from pylbm_isca import regrid as rg
    grads(ref_output)
    basic_state(ref, bs)
    regrid(ref, rg)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
