"""The torch.ops.lbm_gb300 operators are registered with the schemas and fake
(shape) implementations their docstrings give: checked without a device,
under FakeTensorMode, so nothing is launched."""

import pytest

torch = pytest.importorskip("torch")

from lbm_isca_gb300 import ops  # noqa: E402


def _fake():
    from torch._subclasses.fake_tensor import FakeTensorMode
    return FakeTensorMode()


def test_every_operator_is_registered():
    names = set(dir(torch.ops.lbm_gb300))
    for n in ops.OPS:
        assert n in names, n
        assert f"lbm_gb300::{n}" in str(getattr(torch.ops.lbm_gb300, n).default._schema)


def test_transform_operator_shapes():
    L = torch.ops.lbm_gb300
    with _fake():
        f64 = dict(dtype=torch.float64, device="cuda")
        g = torch.empty((3, 64, 128, 5), **f64)
        tw = torch.empty(256, **f64)
        P = torch.empty((43, 43, 64), **f64)
        four = L.fourier_forward(g, None, tw, 42)
        assert four.shape == (3, 43, 64, 5) and four.dtype == torch.complex128
        spec = L.legendre_analysis(four, P, 1, four, P, 0, -1.0, None)
        assert spec.shape == (3, 43, 43, 5)
        back = L.legendre_synthesis(spec, P, 1, None, spec, P, 0, None, 1.0)
        assert back.shape == (3, 43, 64, 5)
        grid = L.fourier_inverse(back, None, tw, 128)
        assert grid.shape == (3, 64, 128, 5) and grid.dtype == torch.float64
        f32 = torch.empty((2, 32, 64, 1), dtype=torch.float32, device="cuda")
        assert L.fourier_forward(f32, None, tw, 21).dtype == torch.complex64


def test_setup_operator_shapes():
    L = torch.ops.lbm_gb300
    with _fake():
        f64 = dict(dtype=torch.float64, device="cuda")
        mu, gw = L.gauss_legendre(torch.empty(0, **f64), 64)
        assert mu.shape == gw.shape == (64,)
        P, H = L.legendre_tables(mu, 42)
        assert P.shape == H.shape == (43, 43, 64)
        assert L.fft_twiddles(mu, 128).shape == (128,)
        mats = L.gravity_wave_matrices(torch.empty(43, **f64), torch.empty((43, 20), **f64),
                                       torch.empty((43, 20), **f64),
                                       torch.empty((20, 20), **f64),
                                       torch.empty((20, 20), **f64), 1200.0)
        assert mats.shape == (43, 20, 20)
        inv, info = L.batched_inverse(mats)
        assert inv.shape == mats.shape and info.shape == (43,) and info.dtype == torch.int32


def test_model_operator_shapes():
    L = torch.ops.lbm_gb300
    with _fake():
        f64 = dict(dtype=torch.float64, device="cuda")
        E, J, I, K = 2, 32, 64, 20
        named = {k: torch.empty(1, **f64) for k in ops.TEND_INPUTS}
        for k in ("u", "v", "t", "q", "vor", "div"):
            named[k] = torch.empty((E, J, I, K), **f64)
        for k in ("pix", "piy", "ps"):
            named[k] = torch.empty((E, J, I), **f64)
        for k in ("frc_t", "frc_ps", "frc_q", "lin_u", "lin_v"):
            named[k] = None
        outs = L.tendency_grid([named[k] for k in ops.TEND_INPUTS], E, J, I, K, 0,
                               [0.286, 0.608, 287.0], [0, 0, 0], True)
        shapes = dict(zip(ops.TEND_OUTPUTS, [tuple(o.shape) for o in outs]))
        assert shapes["fu"] == (E, J, I, K) and shapes["gt_pi"] == (E, J, I)
        assert shapes["omega"] == (E, J, I, K) and shapes["sdot"] == (E, J, I, K + 1)
        c = dict(dtype=torch.complex128, device="cuda")
        lvl = [torch.empty((E, 22, 22, K), **c) for _ in range(4)]
        lvl.insert(3, torch.empty((E, 22, 22), **c))
        new = L.implicit_step([None] * len(ops.IMPL_OPS), lvl, lvl, E, 21, K, 1200.0)
        assert [tuple(x.shape) for x in new] == [tuple(x.shape) for x in lvl]
        adj = L.implicit_step_adjoint([None] * len(ops.IMPL_OPS), lvl, E, 21, K, 1200.0)
        assert len(adj) == 10
        named = {k: None for k in ops.TADJ_INPUTS}
        for k in ops.TADJ_INPUTS[22:]:
            named[k] = torch.empty((E, J, I, K) if k != "a_gt_pi" else (E, J, I), **f64)
        aouts = L.tendency_grid_adjoint([named[k] for k in ops.TADJ_INPUTS], E, J, I, K,
                                        [0.286, 0.608, 287.0])
        assert [tuple(o.shape) for o in aouts] == [(E, J, I, K)] * 6 + [(E, J, I)] * 2
