#!/usr/bin/env python3
"""Generate the golden fixtures by running the reference package itself.

Usage (where the reference checkout is available):

    python tests/golden/make_golden.py <path of the reference checkout>

It imports ``pylbm_isca`` from the given checkout, runs it in FP64 on the
seeded / analytic inputs of ``lbm_isca_gb300.configs`` and writes small
``.npz`` files next to this script.  The fixtures pin the CPU oracle
(``oracle/lbm_oracle.py``) and, through it, the GPU kernels.  Spectral
outputs are stored packed-triangular ([m, n>=m]) to keep the files small.
"""

import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lbm_isca_gb300 import configs  # noqa: E402


def pack(x, M):
    """[..., M, M, (K)] rectangle -> [..., NS, (K)] over n >= m."""
    x = np.asarray(x)
    mm, nn = np.nonzero(np.triu(np.ones((M, M), dtype=bool)))
    if x.shape[-2:] == (M, M):
        return x[..., mm, nn]
    return x[..., mm, nn, :]


def analytic_perturbation(lat, lon, sig, scale=1.0):
    """Smooth deterministic perturbation used for the tendency fixtures."""
    la = np.radians(lat)[:, None, None]
    lo = np.radians(lon)[None, :, None]
    s = np.asarray(sig)[None, None, :]
    c = np.cos(la)
    u = scale * (2.0 * c ** 2 * np.sin(2 * lo) * (1 + s) + 0.5 * np.sin(la) * c * s)
    v = scale * (1.5 * c ** 3 * np.cos(3 * lo + 0.3) * (1.2 - s))
    t = scale * (1.0 * c ** 2 * np.cos(lo - 0.5) * np.sin(np.pi * s) + 0.3 * np.sin(2 * la))
    q = scale * 1e-3 * (c ** 4 * np.sin(lo + 1.0) * s)
    ps = scale * 2.0 * (c[..., 0] ** 2 * np.cos(2 * lo[..., 0] + 0.7))     # hPa
    return u, v, t, q, ps


def main(refdir):
    sys.path.insert(0, refdir)
    sys.path.insert(0, os.path.join(refdir, "analysis"))
    import pylbm_isca as ref
    from pylbm_isca.dynamics import BasicStateTerms, Dynamics
    from pylbm_isca.ensemble import BatchedSpectral, EnsembleForcing
    from pylbm_isca.forcing import SteadyForcing
    from pylbm_isca.state import State
    import tl_verification as tlv

    # ---- A. Gauss nodes and Legendre tables ---------------------------------
    sp21 = ref.Spectral(nlon=64, nlat=32, nmax=21, device="cpu")
    sp42 = ref.Spectral(device="cpu")
    rows = [0, 1, 5, 20, 42]
    np.savez(os.path.join(HERE, "tables.npz"),
             t21_mu=sp21.mu, t21_gw=sp21.gw, t21_P=sp21.pnm, t21_H=sp21.hnm,
             t42_mu=sp42.mu, t42_gw=sp42.gw, t42_rows=np.array(rows),
             t42_P=np.stack([sp42.pnm[m] for m in rows]),
             t42_H=np.stack([sp42.hnm[m] for m in rows]))

    # ---- B. transforms --------------------------------------------------------
    rng = np.random.default_rng(11)
    tr = {}
    for tag, sp, K in (("t21", sp21, 3), ("t42", sp42, 1)):
        M = sp.nmax + 1
        shape_s = (M, M) if K == 1 else (M, M, K)
        shape_g = (sp.nlat, sp.nlon) if K == 1 else (sp.nlat, sp.nlon, K)
        xi = (rng.normal(size=shape_s) + 1j * rng.normal(size=shape_s))
        xi[~sp.mask] = 0.0
        xi[0] = xi[0].real
        chi = (rng.normal(size=shape_s) + 1j * rng.normal(size=shape_s)) * 0.5
        chi[~sp.mask] = 0.0
        chi[0] = chi[0].real
        g1 = rng.normal(size=shape_g)
        g2 = rng.normal(size=shape_g)
        gx, gy = sp.hgrad(xi)
        vor, div = sp.uv_to_vordiv(g1, g2)
        u, v = sp.psichi_to_uv(xi * 1e6, chi * 1e6)
        tr.update({f"{tag}_xi": pack(xi, M), f"{tag}_chi": pack(chi, M),
                   f"{tag}_g1": g1, f"{tag}_g2": g2,
                   f"{tag}_w2g": sp.wave_to_grid(xi),
                   f"{tag}_g2w": pack(sp.grid_to_wave(g1), M),
                   f"{tag}_gx": gx, f"{tag}_gy": gy,
                   f"{tag}_vor": pack(vor, M), f"{tag}_div": pack(div, M),
                   f"{tag}_u": u, f"{tag}_v": v})
    np.savez(os.path.join(HERE, "transforms.npz"), **tr)

    # ---- C. vertical operators -------------------------------------------------
    vt = {}
    for tag, sigm in (("l20", ref.constants.SIGM),
                      ("eq20", configs.equal_sigma_half_levels(20))):
        vg = ref.VerticalGrid(sigm=sigm, device="cpu")
        tbar = 200.0 + 3.0 * np.arange(vg.kmax)
        vg.set_reference_temperature(tbar)
        for name in ("sig", "dsig", "alpha", "dlog2", "dlog3", "cpg", "w3", "wP",
                     "dsigm", "ww", "tbar", "gg", "tmtx", "whmtx", "gcmtx"):
            vt[f"{tag}_{name}"] = np.asarray(getattr(vg, name))
    np.savez(os.path.join(HERE, "vertical.npz"), **vt)

    # ---- D. operators + basic-state terms (T21, equal-sigma L20, plain config) --
    nlon, nlat, nmax = configs.GRIDS["T21"]
    sigm = configs.equal_sigma_half_levels(20)
    sp = ref.Spectral(nlon=nlon, nlat=nlat, nmax=nmax, device="cpu")
    vg = ref.VerticalGrid(sigm=sigm, device="cpu")
    bs = configs.solid_body_basic_state(nlon, nlat, sigm)
    cfg = ref.Config(ndays=1.0, **configs.plain_damping(20))
    m = ref.LBM(bs, sp, vg, cfg)
    m.semi.prepare(cfg.delt)
    bst = m.bst
    ops = dict(kv=m.damping.kv, kd=m.damping.kd, ktt=m.damping.ktt, kq=m.damping.kq,
               semi_m=m.semi.m, semi_minv=m.semi.minv, semi_cond=m.semi.cond,
               tbar=vg.tbar)
    # basic-state terms of the jet state (non-trivial), subsampled grid points
    sub = (slice(None, None, 3), slice(None, None, 5))
    # default-config damping/vdiff on the reference L20 levels
    vgd = ref.VerticalGrid(device="cpu")
    bsd, _ = tlv.load_basic(sp, vgd, path=None)
    md = ref.LBM(bsd, sp, vgd, ref.Config(ndays=1.0))
    md.semi.prepare(600.0)
    md.vdiff.prepare(600.0)
    b = md.bst
    ops.update(jet_tbar=vgd.tbar, jet_vor_g=b.vor_g[sub], jet_div=b.div[sub],
               jet_pix=b.pix[sub], jet_piy=b.piy[sub], jet_sdot=b.sdot[sub],
               jet_x5=b.x5[sub], jet_ssum=b.ssum[sub])
    ops.update(dflt_kv=md.damping.kv, dflt_kd=md.damping.kd,
               dflt_ktt=md.damping.ktt, dflt_kq=md.damping.kq,
               dflt_semi_minv=md.semi.minv, dflt_vd_vor=md.vdiff.minv["vor"],
               dflt_vd_t=md.vdiff.minv["t"])
    np.savez(os.path.join(HERE, "operators_t21.npz"), **ops)

    # ---- E. one tendency call (synthetic jet, default L20 levels, T21) --------
    M = nmax + 1
    u, v, t, q, ps = analytic_perturbation(sp.lat_deg, sp.lon_deg, vgd.sig)
    st = State(np.asarray(bsd.ps), u=u, v=v, t=t, q=q, ps=ps, xp=np)
    ten = {}
    dyn = Dynamics(sp, vgd, md.bst)
    wt = dyn.tendencies(st)
    for name, x in zip(("vor", "div", "t", "pi", "q"), wt):
        ten[name] = pack(x, M)
    ten["omega"] = dyn.diag["omega"][::4, ::4]
    # strictly linear: only the divergence tendency differs (the KE term)
    ten["div_lin"] = pack(Dynamics(sp, vgd, md.bst, strictly_linear=True)
                          .tendencies(st)[1], M)
    # with forcing on every channel
    frc_t = 1e-5 * np.cos(np.radians(sp.lat_deg))[:, None, None] * np.ones((nlat, nlon, 20))
    frc_vor = 1e-11 * np.sin(np.radians(sp.lon_deg))[None, :, None] * np.ones((nlat, nlon, 20))
    frc_div = 2e-11 * np.cos(np.radians(sp.lon_deg))[None, :, None] * np.ones((nlat, nlon, 20))
    frc_ps = 1e-8 * np.cos(np.radians(sp.lat_deg))[:, None] * np.ones((nlat, nlon))
    wt = Dynamics(sp, vgd, md.bst).tendencies(st, frc_t=frc_t, frc_vor=frc_vor,
                                              frc_div=frc_div, frc_ps=frc_ps)
    for name, x in zip(("vor", "div", "t", "pi", "q"), wt):
        ten[f"{name}_frc"] = pack(x, M)
    np.savez(os.path.join(HERE, "tendencies_t21.npz"), **ten)

    # ---- F. short runs ----------------------------------------------------------
    runs = {}

    def save_state(prefix, model, spx, levels=("a", "b")):
        for lvl, stx in ((x, getattr(model, "g" + x)) for x in levels):
            spec = stx.to_spectral(spx)
            for name in ("vor", "div", "t", "pi", "q"):
                runs[f"{prefix}_{lvl}_{name}"] = pack(spec[name], M)
            runs[f"{prefix}_{lvl}_ps"] = np.asarray(stx.ps)

    # F1: plain configuration, solid body, elliptic heating, 40 advancing steps
    heat = configs.elliptic_heating(nlon, nlat, sigm)
    cfg1 = ref.Config(ndays=40 / 72.0, **configs.plain_damping(20))
    m1 = ref.LBM(bs, sp, vg, cfg1)
    frc1 = SteadyForcing(np.zeros_like(heat), np.zeros_like(heat), heat,
                         np.zeros((nlat, nlon)))
    m1.run(steady_forcing=frc1, verbose=False)
    save_state("plain", m1, sp)
    # F2: default configuration (sponge, vdiff, default drag), jet basic state,
    # non-zero initial perturbation, 24 advancing steps
    cfg2 = ref.Config(ndays=24 / 72.0)
    vg2 = ref.VerticalGrid(device="cpu")
    m2 = ref.LBM(bsd, sp, vg2, cfg2)
    ub, vb, tb, qb, psb = analytic_perturbation(sp.lat_deg, sp.lon_deg, vg2.sig, 0.1)
    ub, vb = sp.vordiv_to_uv(*sp.uv_to_vordiv(ub, vb))
    m2.set_initial_perturbation(u=ub, v=vb, t=sp.truncate(tb), q=sp.truncate(qb))
    heat2 = configs.elliptic_heating(nlon, nlat, ref.constants.SIGM, lon0=200.0,
                                     lat0=5.0)
    frc2 = SteadyForcing(np.zeros_like(heat2), np.zeros_like(heat2), heat2,
                         np.zeros((nlat, nlon)))
    m2.run(steady_forcing=frc2, verbose=False)
    save_state("dflt", m2, sp)
    # F3: batched ensemble of 2 members (plain config), 12 advancing steps
    heats, _ = configs.ensemble_heating(nlon, nlat, sigm, 2, seed=1)
    spb = BatchedSpectral(nlon=nlon, nlat=nlat, nmax=nmax, device="cpu")
    cfg3 = ref.Config(ndays=12 / 72.0, nmem=2, **configs.plain_damping(20))
    m3 = ref.LBM(bs, spb, ref.VerticalGrid(sigm=sigm, device="cpu"), cfg3,
                 basic_spectral=sp)
    m3.run(mjo_forcing=EnsembleForcing(heats, np), verbose=False)
    save_state("ens", m3, spb, levels=("a",))
    np.savez_compressed(os.path.join(HERE, "runs_t21.npz"), **runs)

    # ---- G. the reference's own recorded Gill numbers (analysis/gill_isca.json)
    with open(os.path.join(refdir, "analysis", "gill_isca.json")) as fh:
        gill = json.load(fh)
    with open(os.path.join(HERE, "gill_record.json"), "w") as fh:
        json.dump({"source": "analysis/gill_isca.json (reference record)",
                   "experiment": gill["experiment"], "cpu": gill["cpu"]}, fh,
                  indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
