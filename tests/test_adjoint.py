"""Hand-written adjoint of the time step and the checkpointed forcing gradient.

CPU tests: the binomial checkpoint schedule (consistency, stored-state
limit, the binomial bound, which the recursion's exact minimum equals), and
the column arithmetic of the adjoint kernels (adjoint_col.cuh built with
g++) against a numpy restatement of the forward formulas
(dynamics.py:176-267, integrator.py:264-315) by dot products.

GPU tests (FP64): dot products of every transposed transform, of the
tendency, implicit-update and whole-step adjoints against the tangent-linear
model, the tangent-linear tendencies against the reference's own
(``Dynamics(strictly_linear=True)``, golden fixture made by
tests/golden/make_golden_adjoint.py) and the adjoint against it by a dot
product, the tangent-linear tendencies about a non-zero state against
central differences of the reference's nonlinear tendency, the whole-run tangent-linear response against the gradient, the
gradient against central finite differences along 16 seeded directions
(eps = 1e-4 relative), and checkpointing that changes nothing.
"""

import ctypes as C
import os
import shutil
import subprocess
import types

import numpy as np
import pytest

from conftest import ROOT, golden

# ---------------------------------------------------------------- CPU tests


def test_binomial_schedule_meets_the_bound():
    from lbm_isca_gb300.checkpoint import binomial_cost, schedule, simulate

    def exact(t, c, memo={}):
        if t == 1:
            return 0
        if c == 1:
            return t * (t - 1) // 2
        key = (t, c)
        if key not in memo:
            memo[key] = min(l + exact(t - l, c - 1) + exact(l, c) for l in range(1, t))
        return memo[key]

    for t in range(1, 45):
        for c in range(1, 7):
            steps, peak, order = simulate(schedule(t, c))
            assert order == list(range(t - 1, -1, -1))
            assert peak <= c
            assert steps == binomial_cost(t, min(c, t)) == exact(t, min(c, t))
    # 20 days at dt = 1200 s (1440 steps + 2 start-up calls), 32 stored states
    steps, peak, order = simulate(schedule(1442, 32))
    assert peak == 32 and len(order) == 1442 and steps == binomial_cost(1442, 32) == 3731
    # every state stored: one forward sweep, no re-step
    steps, peak, order = simulate(schedule(1442, 1442))
    assert (steps, peak) == (1441, 1442) == (binomial_cost(1442, 1442), 1442)
    assert order == list(range(1441, -1, -1))
    with pytest.raises(ValueError):
        schedule(0, 3)
    with pytest.raises(ValueError):
        simulate([("store", 0), ("advance", 1, 2)])


class _ToyStep:
    """A stand-in for TimeStep on CPU tensors with the same call structure:
    a leapfrog-like nonlinear map of (ga, gb) forced by h, whose exact
    adjoint is written out, so that the gradient driver's bookkeeping (which
    stored state, which next-level ps each adjoint call gets) is checked
    without the GPU."""

    gamma = 0.1

    def __init__(self, torch, shape):
        self.torch, self.shape = torch, shape
        # the heating enters the toy map directly: its transform is the identity
        self.tr = types.SimpleNamespace(grid_to_wave_T=lambda x: x)

    def _state(self, u, v, t, q, ps):
        return types.SimpleNamespace(u=u, v=v, t=t, q=q, ps=ps)

    def _lead(self):
        return ()

    def zero_state(self):
        z = lambda: self.torch.zeros(self.shape, dtype=self.torch.float64)   # noqa: E731
        return self._state(z(), z(), z(), z(), z())

    @staticmethod
    def _c(ga, gb, dt, h):
        # next level: u' = u_b + dt (sin(u_a) + h), ps' = ps_b + dt u_a^2, the
        # other fields carried along linearly
        return (gb.u + dt * (ga.u.sin() + h), gb.v + dt * ga.u, gb.t + dt * ga.v,
                gb.q + 0.5 * ga.t, gb.ps + dt * ga.u * ga.u)

    def forward(self, ga, gb, dt, start, h):
        gc = self._state(*self._c(ga, gb, dt, h))
        if start:
            return gc, ga
        g = self.gamma
        return gc, self._state(*(getattr(ga, k) + g * (getattr(gb, k) - 2 * getattr(ga, k)
                                                       + getattr(gc, k)) for k in
                                 ("u", "v", "t", "q", "ps")))

    def adjoint(self, ga, gb, gc_ps, a_ga, a_gb, dt, start):
        # the map is written as gc = C(ga, gb); gc_ps is checked against it
        assert self.torch.equal(gc_ps, self._c(ga, gb, dt, 0.0)[4])
        keys = ("u", "v", "t", "q", "ps")
        g = self.gamma
        if start:
            ac, aa, ab = a_ga, a_gb, None
        else:
            ac = self._state(*(getattr(a_ga, k) + g * getattr(a_gb, k) for k in keys))
            aa = self._state(*((1 - 2 * g) * getattr(a_gb, k) for k in keys))
            ab = self._state(*(g * getattr(a_gb, k) for k in keys))
        na = self._state(dt * ga.u.cos() * ac.u + dt * ac.v + 2 * dt * ga.u * ac.ps,
                         dt * ac.t, 0.5 * ac.q, 0 * ac.q, 0 * ac.ps)
        nb = self._state(ac.u, ac.v, ac.t, ac.q, ac.ps)
        pa = self._state(*(getattr(na, k) + getattr(aa, k) for k in keys))
        pb = nb if ab is None else self._state(*(getattr(nb, k) + getattr(ab, k) for k in keys))
        return pa, pb, dt * ac.u


def test_auto_stored_states():
    """Every call's state when the trajectory fits the memory share, else as
    many as fit, capped; never fewer than one."""
    pytest.importorskip("torch")
    from lbm_isca_gb300.adjoint import ForcingGradient as FG
    pair = 2 * 64 * 128 * (4 * 20 + 1) * 8           # one T42L20 member, FP64
    assert FG.auto_snaps(1442, pair, 0.5, free_bytes=200 << 30) == 1442
    assert FG.auto_snaps(1442, pair, 0.5, free_bytes=8 << 30) == FG.MAX_SNAPS
    assert FG.auto_snaps(1442, pair, 0.5, free_bytes=100 * pair) == 50
    assert FG.auto_snaps(1442, pair, 0.5, free_bytes=0) == 1


def test_gradient_driver_bookkeeping_on_a_toy_model():
    """The checkpointed gradient of a toy model equals central differences
    and the every-state-stored gradient, for several stored-state counts."""
    torch = pytest.importorskip("torch")
    from lbm_isca_gb300.adjoint import ForcingGradient
    from lbm_isca_gb300.checkpoint import schedule

    shape = (3, 4)
    calls = [(0.025, True), (0.05, True)] + [(0.1, False)] * 13

    class Resp:
        def __call__(self, st):
            return (st.u * st.u).sum() + (st.ps * st.t).sum()

        def seed(self, tr, like):
            z = torch.zeros_like(like.u)
            return types.SimpleNamespace(u=2 * like.u, v=z, t=like.ps, q=z, ps=like.t)

    def driver(snaps):
        fg = ForcingGradient.__new__(ForcingGradient)
        fg.step, fg.response = _ToyStep(torch, shape), Resp()
        fg.use_graph, fg.pipeline, fg._fg, fg._ag = False, False, {}, {}
        fg.calls, fg.snaps = calls, snaps
        fg.actions = schedule(len(calls), snaps)
        fg.forward_steps, fg.peak_stored, fg._saved = 0, 0, None
        fg._heating = lambda h: h
        return fg

    h = torch.as_tensor(np.random.default_rng(8).normal(size=shape))
    ref = None
    for snaps in (1, 2, 3, 5, 15, 40):
        fg = driver(snaps)
        J, g = fg.value_and_grad(h)
        assert fg.peak_stored <= snaps
        if ref is None:
            ref = g
            d = torch.as_tensor(np.random.default_rng(9).normal(size=shape))
            e = 1e-6
            fd = (float(fg.value(h + e * d)) - float(fg.value(h - e * d))) / (2 * e)
            assert abs(fd - float((g * d).sum())) <= 1e-7 * abs(fd)
        else:
            assert torch.allclose(g, ref, rtol=1e-13, atol=0)


def test_response_box_sizes():
    """30-60N x 150-210E: 6 x 11 points at T21, 11 x 21 at T42, 22 x 43 at T85."""
    from lbm_isca_gb300.configs import response_box
    from oracle.lbm_oracle import SphericalTransform
    for (nlon, nlat, nmax), want in (((64, 32, 21), (6, 11)), ((128, 64, 42), (11, 21)),
                                     ((256, 128, 85), (22, 43))):
        tr = SphericalTransform(nlon, nlat, nmax)
        box = response_box(np.degrees(tr.lat), np.degrees(tr.lon))
        assert (int(box.any(axis=1).sum()), int(box.any(axis=0).sum())) == want


@pytest.fixture(scope="module")
def host_adjoint(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("adjcol") / "adjoint_col_host.so")
    src = os.path.join(ROOT, "tests", "adjoint_col_host.cpp")
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-o", out, src])
    return C.CDLL(out)


_D = C.POINTER(C.c_double)


def _p(a):
    return a.ctypes.data_as(_D) if a is not None else None


def _parr(arrs):
    return (_D * len(arrs))(*[_p(a) for a in arrs])


def _column_forward(c, x):
    """Tangent-linear grid-point tendency of one column (dynamics.py:176-267)."""
    from oracle.lbm_oracle import column_sum, sigma_dot, vert_advect
    u, v, t, q, vor, div, pix, piy = x
    padv = u * c["pixb"] + c["ub"] * pix + v * c["piyb"] + c["vb"] * piy
    S = column_sum(div + padv, c["dsig"])
    sd = sigma_dot(S, c["sigm"])
    tv = t + c["eps"] * (t * c["qb"] + c["tb"] * q)
    x5 = c["alpha"] * div + c["wP"] * padv + c["w3"] * S[1:]
    tdev, tvdev = c["tb"] - c["tref"], c["tvb"] - c["tref"]
    rcpg = c["rair"] * c["cpg"]
    va = lambda f, s: vert_advect(f, s, c["dsig"])   # noqa: E731
    gt = (-c["kappa"] * (tv * c["x5b"] + c["tvb"] * x5) + t * c["divb"] + tdev * div
          + va(t, c["sdb"]) + va(c["tb"], sd) + c["tmtx"] @ div)
    fu = (v * c["absv"] + c["vb"] * vor - rcpg * (tv * c["pixb"] + tvdev * pix)
          + va(u, c["sdb"]) + va(c["ub"], sd))
    fv = (-u * c["absv"] - c["ub"] * vor - rcpg * (tv * c["piyb"] + tvdev * piy)
          + va(v, c["sdb"]) + va(c["vb"], sd))
    ke = c["ww"] @ (tv - t) + u * (c["ub"] + c["u0"]) + v * (c["vb"] + c["v0"])
    return [fu, fv, ke, gt, u * tdev + c["ub"] * t, v * tdev + c["vb"] * t,
            q * c["divb"] + c["qb"] * div + va(q, c["sdb"]) + va(c["qb"], sd),
            u * c["qb"] + c["ub"] * q, v * c["qb"] + c["vb"] * q], -(padv * c["dsig"]).sum()


def test_tendency_column_adjoint_is_the_transpose(host_adjoint):
    rng = np.random.default_rng(3)
    K = 7
    r = lambda *s: rng.standard_normal(s)   # noqa: E731
    sigm = np.concatenate([[1.0], np.sort(rng.uniform(0.05, 0.95, K - 1))[::-1], [0.0]])
    sdb = np.concatenate([[0.0], r(K - 1), [0.0]])
    c = dict(dsig=sigm[:-1] - sigm[1:], sigm=sigm, alpha=r(K), w3=r(K), wP=r(K), cpg=r(K),
             ww=r(K, K), tmtx=r(K, K), tref=r(K), ub=r(K), vb=r(K), tb=r(K), qb=r(K),
             tvb=r(K), absv=r(K), divb=r(K), x5b=r(K), sdb=sdb, pixb=0.3, piyb=-0.7,
             kappa=0.2857, eps=0.608, rair=287.04, u0=r(K), v0=r(K))
    x = [r(K) for _ in range(6)] + [0.4, -1.1]
    y = [r(K) for _ in range(9)]
    ypi = 0.9
    out, gtpi = _column_forward(c, x)
    lhs = sum(float(a @ b) for a, b in zip(out, y)) + gtpi * ypi
    vert = [np.ascontiguousarray(c[k]) for k in ("dsig", "sigm", "alpha", "w3", "wP", "cpg",
                                                 "ww", "tmtx", "tref")]
    bs = [np.ascontiguousarray(c[k]) for k in ("ub", "vb", "tb", "qb", "tvb", "absv", "divb",
                                               "x5b", "sdb")]
    aout = [np.zeros(K) for _ in range(6)]
    px, py = C.c_double(), C.c_double()
    work = np.zeros(5 * (K + 1))
    host_adjoint.host_tendency_column_adjoint(
        C.c_int(K), C.c_double(c["kappa"]), C.c_double(c["eps"]), C.c_double(c["rair"]),
        _parr(vert), _parr(bs), C.c_double(c["pixb"]), C.c_double(c["piyb"]), _p(c["u0"]),
        _p(c["v0"]), _parr(y), C.c_double(ypi), _parr(aout), C.byref(px), C.byref(py),
        _p(work))
    rhs = sum(float(a @ b) for a, b in zip(x[:6], aout)) + x[6] * px.value + x[7] * py.value
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def _implicit_forward(c, p, w, n):
    """Semi-implicit update of one coefficient (integrator.py:264-315), real."""
    dt = c["dt"]
    ft = 1.0 + 2.0 * dt * c["ktt"]
    sx = p["t"] * (1.0 + dt * c["ktt"]) + dt * w["t"]
    wdphiy = c["ww"] @ sx + (p["pi"] + dt * w["pi"]) * ft * c["gg"]
    rhs = p["div"] * (1.0 + dt * c["kd"]) * ft + dt * (w["div"] * ft - c["lap"] * wdphiy)
    dbar = c["minv"] @ rhs
    wt2, wpi2 = w["t"] - c["tmtx"] @ dbar, w["pi"] - c["dsig"] @ dbar
    out = {"vor": (p["vor"] + 2 * dt * w["vor"]) / (1 + 2 * dt * c["kv"]),
           "div": 2 * dbar - p["div"], "t": (p["t"] + 2 * dt * wt2) / ft,
           "q": (p["q"] + 2 * dt * w["q"]) / (1 + 2 * dt * c["kq"]),
           "pi": p["pi"] + 2 * dt * wpi2}
    for f, vd in zip(("vor", "div", "t", "q"), c["vd"]):
        if vd is not None and not (f in ("vor", "div") and n < 2):
            out[f] = vd @ out[f]
    return out


@pytest.mark.parametrize("n", [1, 5])
def test_implicit_coefficient_adjoint_is_the_transpose(host_adjoint, n):
    rng = np.random.default_rng(11 + n)
    K = 6
    r = lambda *s: rng.standard_normal(s)   # noqa: E731
    c = dict(dt=1200.0, lap=-n * (n + 1) / 6.371e6 ** 2, kv=abs(r(K)) * 1e-5,
             kd=abs(r(K)) * 1e-5, ktt=abs(r(K)) * 1e-5, kq=abs(r(K)) * 1e-5, ww=r(K, K),
             tmtx=r(K, K), gg=r(K) * 1e4, dsig=abs(r(K)), minv=r(K, K),
             vd=[r(K, K), r(K, K), None, r(K, K)])
    fields = ("vor", "div", "t", "q")
    p = {f: r(K) for f in fields}
    w = {f: r(K) for f in fields}
    p["pi"], w["pi"] = 0.3, -0.8
    y = {f: r(K) for f in fields}
    y["pi"] = 1.7
    out = _implicit_forward(c, p, w, n)
    lhs = sum(float(np.dot(out[f], y[f])) for f in fields) + out["pi"] * y["pi"]
    ops = [np.ascontiguousarray(c[k]) for k in ("kv", "kd", "ktt", "kq", "ww", "tmtx", "gg",
                                                "dsig", "minv")]
    ap, aw = [np.zeros(K) for _ in fields], [np.zeros(K) for _ in fields]
    app, awp = C.c_double(), C.c_double()
    host_adjoint.host_implicit_coef_adjoint(
        C.c_int(K), C.c_double(c["dt"]), C.c_double(c["lap"]), _parr(ops), _parr(c["vd"]),
        C.c_int(int(n < 2)), _parr([y[f] for f in fields]), C.c_double(y["pi"]), _parr(ap),
        C.byref(app), _parr(aw), C.byref(awp), _p(np.zeros(4 * K)))
    rhs = (sum(float(np.dot(p[f], a)) + float(np.dot(w[f], b)) for f, a, b in
               zip(fields, ap, aw)) + p["pi"] * app.value + w["pi"] * awp.value)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


# ---------------------------------------------------------------- GPU tests


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _model(K=20, strictly_linear=False, **extra):
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid, configs
    sigm = configs.equal_sigma_half_levels(K)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    sp = Spectral(nlon=64, nlat=32, nmax=21)
    vg = VerticalGrid(sigm=sigm)
    kw = dict(configs.plain_damping(K), strictly_linear=strictly_linear)
    kw.update(extra)
    cfg = Config(ndays=1.0, **kw)
    return LBM(bs, sp, vg, cfg), sigm


class _Rand:
    def __init__(self, torch, seed, M=22, J=32, I=64, K=20):
        self.t, self.rng, self.M, self.J, self.I, self.K = torch, np.random.default_rng(seed), M, J, I, K

    def grid(self, k=True, scale=1.0):
        shape = (self.J, self.I, self.K) if k else (self.J, self.I)
        return self.t.as_tensor(scale * self.rng.standard_normal(shape)).cuda()

    def spec(self, k=True):
        M = self.M
        shape = (M, M, self.K) if k else (M, M)
        x = self.rng.standard_normal(shape) + 1j * self.rng.standard_normal(shape)
        mask = np.triu(np.ones((M, M), bool))
        return self.t.as_tensor(np.where(mask[..., None] if k else mask, x, 0)).cuda()

    def state(self, step, ps_scale=1.0):
        return step._state(self.grid(), self.grid(), self.grid(), self.grid(scale=1e-3),
                           self.grid(False, ps_scale))


def _rel(a, b):
    return abs(a - b) / max(abs(a), abs(b))


@pytest.mark.gpu
def test_transposed_transforms_dot_products(torch_cuda):
    from lbm_isca_gb300.adjoint import AdjointTransforms, spec_dot
    m, _ = _model()
    sp, tr, r = m.sp, AdjointTransforms(m.sp), _Rand(torch_cuda, 1)
    gd = lambda a, b: float((a * b).sum())   # noqa: E731
    for k in (True, False):
        x, y = r.spec(k), r.grid(k)
        assert _rel(gd(sp.wave_to_grid(x), y), spec_dot(x, tr.wave_to_grid_T(y))) < 1e-13
        g, s = r.grid(k), r.spec(k)
        assert _rel(spec_dot(sp.grid_to_wave(g), s), gd(g, tr.grid_to_wave_T(s))) < 1e-13
    x, gx, gy = r.spec(), r.grid(), r.grid()
    hx, hy = sp.hgrad(x)
    assert _rel(gd(hx, gx) + gd(hy, gy), spec_dot(x, tr.hgrad_T(gx, gy))) < 1e-13
    u, v, s1, s2 = r.grid(), r.grid(), r.spec(), r.spec()
    vo, di = sp.uv_to_vordiv(u, v)
    au, av = tr.uv_to_vordiv_T(s1, s2)
    assert _rel(spec_dot(vo, s1) + spec_dot(di, s2), gd(u, au) + gd(v, av)) < 1e-13
    fx, fy = tr.neg_divergence_T(s1)
    assert _rel(spec_dot(sp.neg_divergence(u, v), s1), gd(u, fx) + gd(v, fy)) < 1e-13
    uu, vv = sp.vordiv_to_uv(s1, s2)
    a1, a2 = tr.vordiv_to_uv_T(u, v)
    assert _rel(gd(uu, u) + gd(vv, v), spec_dot(s1, a1) + spec_dot(s2, a2)) < 1e-13


@pytest.mark.gpu
def test_tendency_and_implicit_adjoints_dot_products(torch_cuda):
    from lbm_isca_gb300.adjoint import TimeStep, spec_dot, state_dot
    m, _ = _model(vdifv=1.0e3, vdifd=1.0e3, vdift=1.0e3, vdifq=2.0e3)
    st, r = TimeStep(m), _Rand(torch_cuda, 2)
    ga, dx = r.state(st), r.state(st)
    aw = [r.spec(), r.spec(), r.spec(), r.spec(False), r.spec()]
    lhs = sum(spec_dot(a, b) for a, b in zip(st.tangent_tendencies(ga, dx), aw))
    assert _rel(lhs, state_dot(dx, st.adjoint_tendencies(ga, aw))) < 1e-12
    keys = ("vor", "div", "t", "pi", "q")
    for dt in (300.0, 1200.0):
        p = {k: r.spec(k != "pi") for k in keys}
        w = [r.spec(k != "pi") for k in keys]
        y = {k: r.spec(k != "pi") for k in keys}
        new = m.integ.step(dt, p, w)
        ap, aw2 = st._implicit_adjoint(dt, y)
        lhs = sum(spec_dot(new[k], y[k]) for k in keys)
        rhs = (sum(spec_dot(p[k], ap[k]) for k in keys)
               + sum(spec_dot(wi, aw2[k]) for wi, k in zip(w, keys)))
        assert _rel(lhs, rhs) < 1e-12


@pytest.mark.gpu
def test_step_forward_matches_the_general_loop(torch_cuda):
    """TimeStep.forward (transforms of one kind batched per call) against
    the model's own reference-sequence step, start-up and leapfrog calls."""
    from lbm_isca_gb300 import configs
    from lbm_isca_gb300.adjoint import FIELDS, TimeStep
    m, sigm = _model()
    st, r = TimeStep(m), _Rand(torch_cuda, 4)
    heat = torch_cuda.as_tensor(configs.elliptic_heating(64, 32, sigm)).cuda()
    ga, gb = r.state(st, 5.0), r.state(st, 5.0)
    for start, dt in ((True, 300.0), (False, 1200.0)):
        gc, gbn = st.forward(ga, gb, dt, start, heat)
        m.ga, m.gb = ga.copy(), gb.copy()
        m._general_step(dt, start, heat, None)
        for k in FIELDS:
            for got, ref in ((getattr(gc, k), getattr(m.ga, k)), (getattr(gbn, k), getattr(m.gb, k))):
                assert float((got - ref).abs().max()) <= 1e-13 * float(ref.abs().max()), k


@pytest.mark.gpu
def test_step_adjoint_dot_product_and_taylor(torch_cuda):
    """Whole step: <TL dx, y> = <dx, ADJ y> to 1e-10 (start-up and leapfrog
    calls), and the TL is the derivative of the nonlinear step."""
    from lbm_isca_gb300.adjoint import FIELDS, TimeStep, state_dot
    m, _ = _model()
    st, r = TimeStep(m), _Rand(torch_cuda, 3)
    ga, gb = r.state(st, 5.0), r.state(st, 5.0)
    dga, dgb = r.state(st), r.state(st)
    for start, dt in ((True, 300.0), (False, 1200.0)):
        gc, _ = st.forward(ga, gb, dt, start, None)
        t1, t2 = st.tangent(ga, gb, gc.ps, dga, dgb, dt, start)
        y1, y2 = r.state(st), r.state(st)
        lhs = state_dot(t1, y1) + state_dot(t2, y2)
        a1, a2, _ = st.adjoint(ga, gb, gc.ps, y1, y2, dt, start)
        assert _rel(lhs, state_dot(dga, a1) + state_dot(dgb, a2)) < 1e-10
        eps = 1e-3
        sh = lambda s, d, e: st._state(*(getattr(s, k) + e * getattr(d, k)   # noqa: E731
                                         for k in FIELDS))
        c1, _ = st.forward(sh(ga, dga, eps), sh(gb, dgb, eps), dt, start, None)
        c2, _ = st.forward(sh(ga, dga, -eps), sh(gb, dgb, -eps), dt, start, None)
        num = sum(float(((getattr(c1, k) - getattr(c2, k)) / (2 * eps)
                         - getattr(t1, k)).abs().max()) for k in FIELDS)
        assert num / sum(float(getattr(t1, k).abs().max()) for k in FIELDS) < 1e-8


@pytest.mark.gpu
def test_adjoint_against_reference_tangent_linear(torch_cuda):
    """The reference's own tangent-linear tendencies (strictly linear
    Dynamics on its synthetic jet and test direction, T21, 5 layers):
    ours reproduce them, and the adjoint is their transpose."""
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid
    from lbm_isca_gb300.adjoint import TimeStep, state_dot
    torch = torch_cuda
    g = golden("adjoint_tl.npz")
    J, I, K = 32, 64, 5
    z3 = lambda p: np.broadcast_to(p[:, None, :], (J, I, K)).copy()   # noqa: E731
    bs = types.SimpleNamespace(u=z3(g["bs_u"]), v=np.zeros((J, I, K)), t=z3(g["bs_t"]),
                               q=z3(g["bs_q"]), ps=np.full((J, I), float(g["bs_ps"])))
    sp, vg = Spectral(nlon=64, nlat=32, nmax=21), VerticalGrid(sigm=g["sigm"])
    m = LBM(bs, sp, vg, Config(strictly_linear=True, sponge=False, ddragv=None, ddragd=None,
                               ddragt=None))
    st = TimeStep(m)
    T = lambda a: torch.as_tensor(np.asarray(a)).cuda()   # noqa: E731
    zero = st.zero_state()
    dx = st._state(T(g["u0"]), T(g["v0"]), T(g["t0"]), T(g["q0"]),
                   T(float(g["bs_ps"]) * g["pi0"]))
    names = ("vor", "div", "t", "pi", "q")
    for n, x in zip(names, st.tangent_tendencies(zero, dx)):
        ref = g["L_" + n]
        assert np.abs(x.cpu().numpy() - ref).max() <= 1e-10 * np.abs(ref).max(), n
    r = _Rand(torch, 7, K=K)
    ys = [r.spec(n != "pi") for n in names]
    lhs = sum(float((np.conj(g["L_" + n]) * y.cpu().numpy()).real.sum())
              for n, y in zip(names, ys))
    rhs = state_dot(dx, st.adjoint_tendencies(zero, ys))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


@pytest.mark.gpu
def test_tangent_linear_about_a_state_against_reference_tendency(torch_cuda):
    """About a non-zero state (the reference's test direction at amplitude
    0.5) the tangent-linear tendencies equal central differences of the
    reference's own nonlinear tendency (kinetic energy kept, exact pi' <->
    ps'), eps = 1e-4, along its second test direction."""
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid
    from lbm_isca_gb300.adjoint import TimeStep
    torch = torch_cuda
    g = golden("adjoint_tl.npz")
    J, I, K = 32, 64, 5
    z3 = lambda p: np.broadcast_to(p[:, None, :], (J, I, K)).copy()   # noqa: E731
    bs = types.SimpleNamespace(u=z3(g["bs_u"]), v=np.zeros((J, I, K)), t=z3(g["bs_t"]),
                               q=z3(g["bs_q"]), ps=np.full((J, I), float(g["bs_ps"])))
    sp, vg = Spectral(nlon=64, nlat=32, nmax=21), VerticalGrid(sigm=g["sigm"])
    m = LBM(bs, sp, vg, Config(strictly_linear=False, sponge=False, ddragv=None,
                               ddragd=None, ddragt=None))
    st = TimeStep(m)
    T = lambda a: torch.as_tensor(np.asarray(a)).cuda()   # noqa: E731
    ps_bar = float(g["bs_ps"])
    x0 = st._state(T(0.5 * g["u0"]), T(0.5 * g["v0"]), T(0.5 * g["t0"]), T(0.5 * g["q0"]),
                   T(ps_bar * (np.exp(0.5 * g["pi0"]) - 1.0)))
    # the reference perturbs pi'; in ps' that is (ps_bar + ps0) d_pi
    dx = st._state(T(g["d_u"]), T(g["d_v"]), T(g["d_t"]), T(g["d_q"]),
                   (st.ps_bar + x0.ps) * T(g["d_pi"]))
    for n, x in zip(("vor", "div", "t", "pi", "q"), st.tangent_tendencies(x0, dx)):
        ref = g["D_" + n]
        assert np.abs(x.cpu().numpy() - ref).max() <= 1e-7 * np.abs(ref).max(), n


@pytest.fixture(scope="module")
def gradient_case(torch_cuda):
    from lbm_isca_gb300 import configs
    from lbm_isca_gb300.adjoint import AreaMeanStreamfunction, ForcingGradient
    m, sigm = _model()
    resp = AreaMeanStreamfunction(m.sp, m.vg)
    assert resp.npts == (6, 11)
    heat = torch_cuda.as_tensor(configs.elliptic_heating(64, 32, sigm)).cuda()
    fg = ForcingGradient(m, resp, nsteps=36, snaps=6)
    J, grad = fg.value_and_grad(heat)
    return types.SimpleNamespace(m=m, resp=resp, heat=heat, fg=fg, J=float(J), grad=grad)


@pytest.mark.gpu
def test_gradient_tangent_linear_run_dot_product(gradient_case, torch_cuda):
    c = gradient_case
    r = _Rand(torch_cuda, 21)
    for _ in range(2):
        d = r.grid() * float(c.heat.abs().max())
        tl = float(c.fg.tangent(c.heat, d))
        assert _rel(tl, float((c.grad * d).sum())) < 1e-10


@pytest.mark.gpu
def test_gradient_matches_central_differences(gradient_case, torch_cuda):
    """16 seeded random directions, eps = 1e-4 relative to the heating."""
    c = gradient_case
    assert abs(c.J - float(c.fg.value(c.heat))) <= 1e-12 * abs(c.J)
    rng = np.random.default_rng(16)
    hmax = float(c.heat.abs().max())
    worst = 0.0
    for _ in range(16):
        d = torch_cuda.as_tensor(rng.standard_normal(tuple(c.heat.shape))).cuda() * hmax
        eps = 1e-4
        fd = (float(c.fg.value(c.heat + eps * d)) - float(c.fg.value(c.heat - eps * d))) / (2 * eps)
        worst = max(worst, _rel(fd, float((c.grad * d).sum())))
    assert worst < 1e-6


@pytest.mark.gpu
def test_checkpointing_changes_nothing(gradient_case, torch_cuda):
    from lbm_isca_gb300.adjoint import ForcingGradient, HeatingResponse
    c = gradient_case
    assert c.fg.peak_stored <= 6
    # eager calls with every state stored against graph replays from 6
    # stored states: the same kernels in the same order
    full = ForcingGradient(c.m, c.resp, nsteps=36, snaps=64, use_graph=False)
    J2, g2 = full.value_and_grad(c.heat)
    assert abs(float(J2) - c.J) <= 1e-13 * abs(c.J)
    assert float((g2 - c.grad).abs().max()) <= 1e-13 * float(c.grad.abs().max())
    assert full.forward_steps == len(full.calls)       # every state stored: no re-steps
    # every state stored, two streams against one: the reverse sweep's
    # hand-over ring must not race with its own initialisation
    for pipe in (True, False):
        g = ForcingGradient(c.m, c.resp, nsteps=6, snaps=32, pipeline=pipe).value_and_grad(
            c.heat)[1]
        if pipe:
            g_pipe = g
    assert bool((g_pipe == g).all())
    h = c.heat.clone().requires_grad_(True)
    HeatingResponse.apply(h, ForcingGradient(c.m, c.resp, nsteps=36, snaps=3)).backward()
    assert float((h.grad - c.grad).abs().max()) <= 1e-13 * float(c.grad.abs().max())


@pytest.mark.gpu
def test_batched_gradient_matches_single_members(torch_cuda):
    """E members with their own heatings reversed together: each member's J
    and gradient equal its own single-member run; the tangent-linear
    response of each member equals its gradient's dot product."""
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid, configs
    from lbm_isca_gb300.adjoint import AreaMeanStreamfunction, ForcingGradient
    from lbm_isca_gb300.ensemble import make_ensemble_model
    torch = torch_cuda
    K, E = 20, 3
    sigm = configs.equal_sigma_half_levels(K)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    heats = torch.as_tensor(configs.ensemble_heating(64, 32, sigm, E, seed=4)[0]).cuda()
    mk = lambda: Config(ndays=1.0, **configs.plain_damping(K))   # noqa: E731
    mb, spb, vgb = make_ensemble_model(bs, E, mk(), device="cuda", nlon=64, nlat=32, nmax=21,
                                       sigm=sigm)
    fb = ForcingGradient(mb, AreaMeanStreamfunction(spb, vgb), nsteps=24, snaps=5)
    Jb, gb = fb.value_and_grad(heats)
    assert tuple(Jb.shape) == (E,) and tuple(gb.shape) == tuple(heats.shape)
    sp, vg = Spectral(nlon=64, nlat=32, nmax=21), VerticalGrid(sigm=sigm)
    m1 = LBM(bs, sp, vg, mk())
    for e in range(E):
        J1, g1 = ForcingGradient(m1, AreaMeanStreamfunction(sp, vg), nsteps=24,
                                 snaps=5).value_and_grad(heats[e])
        assert abs(float(J1) - float(Jb[e])) <= 1e-12 * abs(float(J1))
        assert float((g1 - gb[e]).abs().max()) <= 1e-12 * float(g1.abs().max())
    d = torch.as_tensor(np.random.default_rng(2).normal(size=tuple(heats.shape))).cuda()
    tl = fb.tangent(heats, d * float(heats.abs().max()))
    dots = (gb * d * float(heats.abs().max())).sum(dim=(1, 2, 3))
    assert float(((tl - dots).abs() / dots.abs()).max()) < 1e-10


@pytest.mark.gpu
def test_fp32_step_adjoint_dot_product(torch_cuda):
    """The FP32 step: forward within 1e-4 (of each field's largest value) of
    the FP64 step, and <TL dx, y> = <dx, ADJ y> to 1e-3 (start-up and
    leapfrog calls)."""
    from lbm_isca_gb300.adjoint import FIELDS, TimeStep, state_dot
    m, _ = _model()
    s64, s32 = TimeStep(m), TimeStep(m, "fp32")
    r = _Rand(torch_cuda, 5)
    f32 = lambda st: s32._state(*(getattr(st, k).float() for k in FIELDS))   # noqa: E731
    ga, gb = r.state(s64, 5.0), r.state(s64, 5.0)
    dga, dgb = r.state(s64), r.state(s64)
    for start, dt in ((True, 300.0), (False, 1200.0)):
        gc, gbn = s64.forward(ga, gb, dt, start, None)
        gc32, gbn32 = s32.forward(f32(ga), f32(gb), dt, start, None)
        for k in FIELDS:
            for a, b in ((getattr(gc32, k), getattr(gc, k)), (getattr(gbn32, k), getattr(gbn, k))):
                assert a.dtype == torch_cuda.float32
                assert float((a.double() - b).abs().max()) <= 1e-4 * float(b.abs().max()), k
        t1, t2 = s32.tangent(f32(ga), f32(gb), gc32.ps, f32(dga), f32(dgb), dt, start)
        y1, y2 = f32(r.state(s64)), f32(r.state(s64))
        lhs = state_dot(t1, y1) + state_dot(t2, y2)
        a1, a2, _ = s32.adjoint(f32(ga), f32(gb), gc32.ps, y1, y2, dt, start)
        assert all(getattr(a1, k).dtype == torch_cuda.float32 for k in FIELDS)
        rhs = state_dot(f32(dga), a1) + state_dot(f32(dgb), a2)
        assert _rel(lhs, rhs) < 1e-3, (lhs, rhs)


@pytest.mark.gpu
def test_fp32_gradient_against_fp64(gradient_case, torch_cuda):
    """The FP32 checkpointed gradient over 36 calls against the FP64 one."""
    from lbm_isca_gb300.adjoint import AreaMeanStreamfunction, ForcingGradient
    c = gradient_case
    fg = ForcingGradient(c.m, None, nsteps=36, precision="fp32")
    fg.response = AreaMeanStreamfunction(fg.step.sp, c.m.vg)
    J, g = fg.value_and_grad(c.heat)
    assert g.dtype == torch_cuda.float32
    assert fg.forward_steps == len(fg.calls)
    assert abs(float(J) - c.J) <= 1e-5 * abs(c.J), (float(J), c.J)
    assert float((g.double() - c.grad).abs().max()) <= 1e-4 * float(c.grad.abs().max())
