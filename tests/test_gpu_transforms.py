"""GPU parity of the spectral transforms against the oracle and the golden
vectors, plus the reference's own analytic transform checks
(tests/test_spectral.py of the reference) re-run on the GB300 path."""

import numpy as np
import pytest

from conftest import golden, pack, relerr, unpack
from oracle import lbm_oracle as orc

pytestmark = pytest.mark.gpu

GRIDS = {"T21": (64, 32, 21), "T42": (128, 64, 42), "T85": (256, 128, 85)}


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _sp(tag, precision="fp64"):
    from lbm_isca_gb300.spectral import Spectral
    nlon, nlat, nmax = GRIDS[tag]
    return Spectral(nlon=nlon, nlat=nlat, nmax=nmax, device="gb300", precision=precision)


def _np(x):
    return x.detach().cpu().numpy()


@pytest.mark.parametrize("tag", ["T21", "T42", "T85"])
def test_gauss_and_tables(torch_cuda, tag):
    sp = _sp(tag)
    tr = orc.SphericalTransform(*GRIDS[tag])
    assert relerr(sp.mu, tr.mu) < 1e-14
    # Newton weights here are ~6e-15 from exact (mpmath) at 128 latitudes,
    # numpy's leggauss (the reference's) ~2.6e-13: compare at 5e-13.
    assert relerr(sp.gw, tr.gw) < 5e-13
    assert abs(sp.gw.sum() - 1.0) < 1e-13
    assert relerr(_np(sp.pnm), tr.P) < 1e-12
    assert relerr(_np(sp.hnm), tr.H) < 1e-12


def test_tables_against_golden(torch_cuda):
    g = golden("tables.npz")
    sp = _sp("T21")
    assert relerr(sp.mu, g["t21_mu"]) < 1e-14
    assert relerr(_np(sp.pnm), g["t21_P"]) < 1e-12
    assert relerr(_np(sp.hnm), g["t21_H"]) < 1e-12


@pytest.mark.parametrize("tag,K", [("T21", 3), ("T42", 1), ("T85", 2)])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 2e-5)])
def test_transforms_vs_oracle(torch_cuda, tag, K, precision, tol):
    sp = _sp(tag, precision)
    tr = orc.SphericalTransform(*GRIDS[tag])
    M = tr.nmax + 1
    rng = np.random.default_rng(5)
    sshape = (M, M) if K == 1 else (M, M, K)
    gshape = (tr.nlat, tr.nlon) if K == 1 else (tr.nlat, tr.nlon, K)
    xi = rng.normal(size=sshape) + 1j * rng.normal(size=sshape)
    xi[~tr.mask] = 0.0
    xi[0] = xi[0].real
    chi = rng.normal(size=sshape) + 1j * rng.normal(size=sshape)
    chi[~tr.mask] = 0.0
    chi[0] = chi[0].real
    g1 = rng.normal(size=gshape)
    g2 = rng.normal(size=gshape)
    assert relerr(_np(sp.wave_to_grid(xi)), tr.wave_to_grid(xi)) < tol
    assert relerr(_np(sp.grid_to_wave(g1)), tr.grid_to_wave(g1)) < tol
    gx, gy = sp.hgrad(xi)
    ox, oy = tr.hgrad(xi)
    assert relerr(_np(gx), ox) < tol and relerr(_np(gy), oy) < tol
    vor, div = sp.uv_to_vordiv(g1, g2)
    ov, od = tr.uv_to_vordiv(g1, g2)
    assert relerr(_np(vor), ov) < tol and relerr(_np(div), od) < tol
    u, v = sp.psichi_to_uv(xi * 1e6, chi * 1e6)
    ou, ovv = tr.psichi_to_uv(xi * 1e6, chi * 1e6)
    assert relerr(_np(u), ou) < tol and relerr(_np(v), ovv) < tol
    u2, v2 = sp.vordiv_to_uv(xi * 1e-5, chi * 1e-5)
    ou2, ov2 = tr.vordiv_to_uv(xi * 1e-5, chi * 1e-5)
    assert relerr(_np(u2), ou2) < tol and relerr(_np(v2), ov2) < tol


@pytest.mark.parametrize("tag", ["t21", "t42"])
def test_transforms_vs_golden(torch_cuda, tag):
    g = golden("transforms.npz")
    sp = _sp(tag.upper())
    M = sp.nmax + 1
    xi = unpack(g[f"{tag}_xi"], M)
    chi = unpack(g[f"{tag}_chi"], M)
    assert relerr(_np(sp.wave_to_grid(xi)), g[f"{tag}_w2g"]) < 1e-12
    assert relerr(pack(_np(sp.grid_to_wave(g[f"{tag}_g1"])), M), g[f"{tag}_g2w"]) < 1e-12
    gx, gy = sp.hgrad(xi)
    assert relerr(_np(gx), g[f"{tag}_gx"]) < 1e-12
    assert relerr(_np(gy), g[f"{tag}_gy"]) < 1e-12
    vor, div = sp.uv_to_vordiv(g[f"{tag}_g1"], g[f"{tag}_g2"])
    assert relerr(pack(_np(vor), M), g[f"{tag}_vor"]) < 1e-12
    assert relerr(pack(_np(div), M), g[f"{tag}_div"]) < 1e-12
    u, v = sp.psichi_to_uv(xi * 1e6, chi * 1e6)
    assert relerr(_np(u), g[f"{tag}_u"]) < 1e-12
    assert relerr(_np(v), g[f"{tag}_v"]) < 1e-12


def test_batched_transforms_match_single(torch_cuda):
    """BatchedSpectral (member axis) == per-member Spectral (ensemble.py:41-106)."""
    from lbm_isca_gb300.ensemble import BatchedSpectral
    sp = _sp("T21")
    bsp = BatchedSpectral(nlon=64, nlat=32, nmax=21, device="gb300")
    rng = np.random.default_rng(9)
    g = rng.normal(size=(3, 32, 64, 4))
    xb = _np(bsp.grid_to_wave(g))
    for e in range(3):
        assert relerr(xb[e], _np(sp.grid_to_wave(g[e]))) < 1e-14
    s2 = rng.normal(size=(3, 32, 64))
    x2 = _np(bsp.grid_to_wave(s2))
    for e in range(3):
        assert relerr(x2[e], _np(sp.grid_to_wave(s2[e]))) < 1e-14


# ---- the reference's analytic transform checks (its tests/test_spectral.py)
def test_ref_legendre_orthonormality(torch_cuda):
    sp = _sp("T42")
    P = _np(sp.pnm)
    worst = 0.0
    for m in [0, 1, 5, 20, 42]:
        p = P[m, m:]
        gram = (p * sp.gw) @ p.T
        worst = max(worst, np.abs(gram - np.eye(gram.shape[0])).max())
    assert worst < 1e-10


def test_ref_roundtrip_and_laplacian(torch_cuda):
    sp = _sp("T42")
    rng = np.random.default_rng(0)
    xi = np.zeros((43, 43), dtype=complex)
    xi[sp.mask] = rng.normal(size=sp.mask.sum()) + 1j * rng.normal(size=sp.mask.sum())
    xi[0] = xi[0].real
    xi2 = _np(sp.grid_to_wave(sp.wave_to_grid(xi)))
    assert np.abs(xi2 - xi)[sp.mask].max() / np.abs(xi)[sp.mask].max() < 1e-11
    for (m, n) in [(0, 1), (1, 1), (3, 7), (10, 20)]:
        x = np.zeros((43, 43), dtype=complex)
        x[m, n] = 1.0 + 0.5j
        g = _np(sp.wave_to_grid(x))
        lap = _np(sp.wave_to_grid(sp.laplacian(x)))
        expect = -n * (n + 1) / sp.a ** 2 * g
        assert np.abs(lap - expect).max() / np.abs(expect).max() < 1e-10


def test_ref_gradients_and_solid_body(torch_cuda):
    sp = _sp("T42")
    f = np.repeat(sp.mu[:, None], sp.nlon, axis=1)
    dfdx, dfdy = sp.hgrad(sp.grid_to_wave(f))
    assert np.abs(_np(dfdx)).max() < 1e-16
    expect = np.sqrt(1 - sp.mu ** 2)[:, None] / sp.a
    assert np.abs(_np(dfdy) - expect).max() / expect.max() < 1e-10
    lam = sp.lon[None, :]
    cl = np.sqrt(1 - sp.mu ** 2)[:, None]
    dfdx, dfdy = sp.hgrad(sp.grid_to_wave(np.cos(lam) * cl))
    ex = -np.sin(lam) / sp.a * np.ones_like(cl)
    ey = -np.cos(lam) * sp.mu[:, None] / sp.a
    assert np.abs(_np(dfdx) - ex).max() / np.abs(ex).max() < 1e-10
    assert np.abs(_np(dfdy) - ey).max() / np.abs(ey).max() < 1e-10
    u = 20.0 * cl * np.ones((1, sp.nlon))
    vor, div = sp.uv_to_vordiv(u, np.zeros_like(u))
    zg = _np(sp.wave_to_grid(vor))
    assert np.abs(_np(sp.wave_to_grid(div))).max() < 1e-18
    ez = 2.0 * 20.0 * sp.mu[:, None] / sp.a
    assert np.abs(zg - ez).max() / np.abs(ez).max() < 1e-10


def test_ref_vordiv_roundtrip_and_div_grad(torch_cuda):
    sp = _sp("T42")
    rng = np.random.default_rng(1)
    xi = np.zeros((43, 43), dtype=complex)
    sel = sp.mask.copy()
    sel[:, 0] = False
    xi[sel] = rng.normal(size=sel.sum()) + 1j * rng.normal(size=sel.sum())
    xi[0] = xi[0].real
    psi, chi = xi * 1e6, xi.conj() * 5e5
    chi[0] = chi[0].real
    u, v = sp.psichi_to_uv(psi, chi)
    vor, div = sp.uv_to_vordiv(u, v)
    psi2 = _np(sp.inverse_laplacian(vor))
    chi2 = _np(sp.inverse_laplacian(div))
    assert np.abs(psi2 - psi)[sel].max() / np.abs(psi)[sel].max() < 1e-10
    assert np.abs(chi2 - chi)[sel].max() / np.abs(chi)[sel].max() < 1e-10
    rng = np.random.default_rng(2)
    xi = np.zeros((43, 43), dtype=complex)
    sel = sp.mask.copy()
    sel[:, 41:] = False
    xi[sel] = rng.normal(size=sel.sum()) + 1j * rng.normal(size=sel.sum())
    xi[0] = xi[0].real
    gx, gy = sp.hgrad(xi)
    divg = -_np(sp.neg_divergence(gx, gy))
    lap = _np(sp.laplacian(xi))
    assert np.abs(divg - lap)[sel].max() / np.abs(lap)[sel].max() < 1e-9


def test_ref_multilevel_consistency(torch_cuda):
    sp = _sp("T42")
    f = np.random.default_rng(3).normal(size=(64, 128, 4))
    xi3 = _np(sp.grid_to_wave(f))
    for k in range(4):
        assert np.abs(xi3[:, :, k] - _np(sp.grid_to_wave(f[:, :, k]))).max() < 1e-12
