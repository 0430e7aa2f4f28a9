"""Every torch.ops.lbm_gb300 operator called through torch.ops on the GPU and
checked against the numpy oracle (or, for the adjoint operators, which have
no reference counterpart, against the tangent-linear model by the
dot-product identity).  A dispatch-mode log also checks that the package's
classes reach the library through these operators."""

import types

import numpy as np
import pytest

from conftest import relerr
from oracle import lbm_oracle as orc
from lbm_isca_gb300 import configs, ops

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def _np(x):
    return x.detach().cpu().numpy()


class OpLog:
    """Records the lbm_gb300 operators dispatched inside a `with` block."""

    def __init__(self, torch):
        from torch.utils._python_dispatch import TorchDispatchMode
        log = self.names = set()

        class Mode(TorchDispatchMode):
            def __torch_dispatch__(self, func, types, args=(), kwargs=None):
                name = str(func)
                if name.startswith("lbm_gb300."):
                    log.add(name.split(".")[1])
                return func(*args, **(kwargs or {}))

        self.mode = Mode()

    def __enter__(self):
        self.mode.__enter__()
        return self

    def __exit__(self, *exc):
        return self.mode.__exit__(*exc)


def test_setup_operators_vs_oracle(torch):
    L = torch.ops.lbm_gb300
    f64 = dict(dtype=torch.float64, device="cuda")
    tr = orc.SphericalTransform(128, 64, 42)
    mu, gw = L.gauss_legendre(torch.empty(0, **f64), 64)
    assert relerr(_np(mu), tr.mu) < 1e-14 and relerr(_np(gw), tr.gw) < 5e-13
    P, H = L.legendre_tables(mu, 42)
    assert relerr(_np(P), tr.P) < 1e-12 and relerr(_np(H), tr.H) < 1e-12
    tw = L.fft_twiddles(mu, 128)
    assert relerr(_np(tw), np.exp(-2j * np.pi * np.arange(128) / 128)) < 1e-15
    lv = orc.SigmaLevels(configs.equal_sigma_half_levels(20))
    lv.set_reference_temperature(np.full(20, 250.0))
    pd = configs.plain_damping(20)
    dmp = orc.DampingCoefs(42, lv, order=pd["hdif_order"], tefold=pd["hdif_tefold"],
                           tunit_hdif=pd["hdif_tunit"], ddragv=pd["ddragv"],
                           ddragd=pd["ddragd"], ddragt=pd["ddragt"], sponge=pd["sponge"])
    args = [torch.as_tensor(x, **f64) for x in (tr.lap, dmp.ktt, dmp.kd, lv.whmtx, lv.gcmtx)]
    mats = L.gravity_wave_matrices(*args, 1200.0)
    ref = orc.gravity_wave_matrices(1200.0, tr.lap, dmp.ktt, dmp.kd, lv.whmtx, lv.gcmtx)
    assert relerr(_np(mats), ref) < 1e-14
    inv, info = L.batched_inverse(mats)
    assert int(info.abs().max()) == 0
    assert relerr(_np(inv), np.linalg.inv(ref)) < 1e-12


@pytest.mark.parametrize("dtype,tol", [("float64", 1e-12), ("float32", 2e-5)])
def test_transform_operators_vs_oracle(torch, dtype, tol):
    L = torch.ops.lbm_gb300
    rd = getattr(torch, dtype)
    cd = torch.complex128 if dtype == "float64" else torch.complex64
    tr = orc.SphericalTransform(64, 32, 21)
    rng = np.random.default_rng(7)
    g = rng.normal(size=(32, 64, 3))
    dev = dict(device="cuda")
    P = torch.as_tensor(tr.P, **dev).to(rd)
    Pgw = torch.as_tensor(tr.P_gw, **dev).to(rd)
    H = torch.as_tensor(tr.H, **dev).to(rd)
    tw = torch.view_as_real(L.fft_twiddles(torch.empty(0, **dev), 64)).reshape(-1).to(rd)
    four = L.fourier_forward(torch.as_tensor(g, **dev).to(rd)[None], None, tw, 21)
    assert relerr(_np(four[0]), tr.fourier_fwd(g)) < tol
    spec = L.legendre_analysis(four, Pgw, 0, None, None, 0, 1.0, None)
    assert relerr(_np(spec[0]), tr.grid_to_wave(g)) < tol
    xi = tr.grid_to_wave(g)
    four2 = L.legendre_synthesis(torch.as_tensor(xi, **dev).to(cd)[None], P, 0, None, None, None, 0,
                                 None, 1.0)
    back = L.fourier_inverse(four2, None, tw, 64)
    assert relerr(_np(back[0]), tr.wave_to_grid(xi)) < tol
    # the gradient pair (i m P and H tables, 1/(a cos) latitude scale)
    rc = torch.as_tensor(1.0 / (tr.a * tr.coslat), **dev).to(rd)
    gx = L.fourier_inverse(L.legendre_synthesis(torch.as_tensor(xi, **dev).to(cd)[None], P, 1, None,
                                                None, None, 0, None, 1.0), rc, tw, 64)
    gy = L.fourier_inverse(L.legendre_synthesis(torch.as_tensor(xi, **dev).to(cd)[None], H, 0, None,
                                                None, None, 0, None, 1.0), rc, tw, 64)
    ox, oy = tr.hgrad(xi)
    assert relerr(_np(gx[0]), ox) < tol and relerr(_np(gy[0]), oy) < tol
    # analysis with two terms (uv_to_vordiv's vorticity: i m P gwdel Fv + H gwdel Fu)
    u, v = rng.normal(size=(2, 32, 64, 3))
    c = torch.as_tensor(tr.coslat, **dev).to(rd)
    Fu = L.fourier_forward(torch.as_tensor(u, **dev).to(rd)[None], c, tw, 21)
    Fv = L.fourier_forward(torch.as_tensor(v, **dev).to(rd)[None], c, tw, 21)
    vor = L.legendre_analysis(Fv, torch.as_tensor(tr.P_gwdel, **dev).to(rd), 1, Fu,
                              torch.as_tensor(tr.H_gwdel, **dev).to(rd), 0, 1.0, None)
    assert relerr(_np(vor[0]), tr.uv_to_vordiv(u, v)[0]) < tol


def _t21_model(torch, precision="fp64", nmem=None, ndays=6 / 72.0):
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid
    from lbm_isca_gb300.ensemble import make_ensemble_model
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    cfg = Config(ndays=ndays, precision=precision, **configs.plain_damping(20))
    if nmem:
        m, _, _ = make_ensemble_model(bs, nmem, cfg, device="gb300", nlon=64, nlat=32,
                                      nmax=21, sigm=sigm)
        return m, bs, sigm
    sp = Spectral(nlon=64, nlat=32, nmax=21, device="gb300")
    return LBM(bs, sp, VerticalGrid(sigm=sigm, device="gb300"), cfg), bs, sigm


def test_model_operators_vs_oracle(torch):
    """Dynamics.tendencies (tendency_grid), Integrator.step (implicit_step)
    and the general and fused loops against the oracle, with the operators
    each dispatches."""
    m, bs, sigm = _t21_model(torch)
    tr = orc.SphericalTransform(64, 32, 21)
    lv = orc.SigmaLevels(sigm)
    om = orc.OracleModel(tr, lv, bs, orc.RunConfig(**configs.plain_damping(20)))
    heat = configs.elliptic_heating(64, 32, sigm)
    rng = np.random.default_rng(3)
    u, v = tr.vordiv_to_uv(*tr.uv_to_vordiv(*rng.normal(size=(2, 32, 64, 20))))
    st = types.SimpleNamespace(u=u, v=v, t=tr.wave_to_grid(tr.grid_to_wave(
        rng.normal(size=(32, 64, 20)))), q=np.zeros((32, 64, 20)),
        ps=0.5 * tr.wave_to_grid(tr.grid_to_wave(rng.normal(size=(32, 64)))))
    from lbm_isca_gb300.state import State
    gst = State(bs.ps, u=st.u, v=st.v, t=st.t, q=st.q, ps=st.ps, device="gb300")
    ost = orc.GridState(np.asarray(bs.ps), st.u, st.v, st.t, st.q, st.ps)
    with OpLog(torch) as log:
        got = m.dyn.tendencies(gst, frc_t=heat)
        prev = gst.to_spectral(m.sp)
        new = m.integ.step(1200.0, prev, got)
    ref = orc.tendencies(tr, lv, om.bt, ost, frc_t=heat)
    for a, b in zip(got, ref):
        assert relerr(_np(a), b) < 1e-10
    oprev = ost.to_spectral(tr)
    onew = om.implicit_step(1200.0, oprev, ref)
    for k in ("vor", "div", "t", "pi", "q"):
        assert relerr(_np(new[k]), onew[k]) < 1e-10, k
    assert {"tendency_grid", "implicit_step", "fourier_forward", "fourier_inverse",
            "legendre_analysis", "legendre_synthesis"} <= log.names
    # the fused stepper from the zero state, 6 steps, against the oracle
    sf = types.SimpleNamespace(t=heat, vor=None, div=None, ps=None)
    with OpLog(torch) as log2:
        m.run(steady_forcing=sf, verbose=False)
    om.run(nsteps=6, frc_t=heat)
    for k in ("u", "v", "t", "ps"):
        assert relerr(_np(getattr(m.ga, k)), getattr(om.ga, k)) < 1e-10, k
    assert {"stepper_prime", "stepper_run", "stepper_flush"} <= log2.names


def test_stepper_and_history_operators(torch):
    """The stepper operators of a fused run from a non-zero state
    (stepper_colsum after loading it) and of a fused run with a history
    writer (history_accumulate), each against the general loop."""
    outs = {}
    for fused in (True, False):
        m, bs, sigm = _t21_model(torch)
        m.cfg.fused = fused
        heat = configs.elliptic_heating(64, 32, sigm)
        sf = types.SimpleNamespace(t=heat, vor=None, div=None, ps=None)

        class W:
            def __init__(self):
                self.days = []

            def add(self, day, fields):
                self.days.append({k: np.array(v) for k, v in fields.items()})

            def close(self):
                pass
        w = W()
        m.cfg.ndays = 1.0
        with OpLog(torch) as log1:
            m.run(steady_forcing=sf, writer=w, verbose=False)     # from the zero state
        m.cfg.ndays = 6 / 72.0
        with OpLog(torch) as log2:
            m.run(steady_forcing=sf, verbose=False)               # from a non-zero state
        outs[fused] = (m, w.days, log1.names, log2.names)
    (mf, df, n1, n2), (mg, dg, _, _) = outs[True], outs[False]
    assert {"history_accumulate", "stepper_run"} <= n1
    assert {"stepper_colsum", "stepper_prime", "stepper_run"} <= n2
    for k in ("u", "v", "t", "ps"):
        assert relerr(_np(getattr(mf.ga, k)), _np(getattr(mg.ga, k))) < 1e-10, k
    assert len(df) == len(dg) == 1
    for k in df[0]:
        assert relerr(df[0][k], dg[0][k]) < 1e-9, k


def test_adjoint_operators_dot_product(torch):
    """tendency_grid_adjoint and implicit_step_adjoint through torch.ops: the
    adjoint of one call against its tangent-linear model (no reference
    counterpart; the identity <TL d, y> = <d, AD y> to 1e-10)."""
    from lbm_isca_gb300.adjoint import TimeStep, state_dot
    m, bs, sigm = _t21_model(torch)
    st = TimeStep(m)
    rng = np.random.default_rng(11)

    def rs():
        t = lambda *s: torch.as_tensor(rng.normal(size=s), device="cuda")   # noqa: E731
        return st._state(t(32, 64, 20), t(32, 64, 20), t(32, 64, 20), t(32, 64, 20) * 1e-3,
                         t(32, 64))
    ga, gb, da, db, ya, yb = rs(), rs(), rs(), rs(), rs(), rs()
    gc, _ = st.forward(ga, gb, 1200.0, False, None)
    with OpLog(torch) as log:
        t1, t2 = st.tangent(ga, gb, gc.ps, da, db, 1200.0, False)
        a1, a2, _ = st.adjoint(ga, gb, gc.ps, ya, yb, 1200.0, False)
    lhs = state_dot(t1, ya) + state_dot(t2, yb)
    rhs = state_dot(da, a1) + state_dot(db, a2)
    assert abs(lhs - rhs) / abs(lhs) < 1e-10
    assert {"tendency_grid_adjoint", "implicit_step_adjoint", "tendency_grid"} <= log.names


@pytest.mark.parametrize("n", [1, 13, 4096, 1000003])
def test_link_copy_round_trip(torch, n):
    """lbm_link_copy (link_copy_): pinned host -> device -> pinned host, any
    length, bit for bit; pageable host memory is refused."""
    src = torch.arange(n, dtype=torch.float64).mul_(1.0 / 3.0).pin_memory()
    dev = torch.empty(n, dtype=torch.float64, device="cuda")
    back = torch.empty(n, dtype=torch.float64).pin_memory()
    torch.ops.lbm_gb300.link_copy_(dev, src)
    torch.ops.lbm_gb300.link_copy_(back, dev)
    torch.cuda.synchronize()
    assert torch.equal(back, src)
    assert torch.equal(dev.cpu(), src)
    b8 = torch.arange(n, dtype=torch.uint8).pin_memory()
    d8 = torch.empty(n, dtype=torch.uint8, device="cuda")
    torch.ops.lbm_gb300.link_copy_(d8, b8)
    torch.cuda.synchronize()
    assert torch.equal(d8.cpu(), b8)
    with pytest.raises(ValueError):
        torch.ops.lbm_gb300.link_copy_(torch.empty(n, dtype=torch.float64), dev)
