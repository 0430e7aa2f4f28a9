"""The plain single-member configuration at T42L20 against the reference's
own trajectory: the FP64 path to 1e-10 and the FP32 path to 1e-5 relative L2
per prognostic field, after 10 and 30 model days (722 and 2162 calls of the
step, model.py:213-247).

Golden: tests/golden/t42l20_reference_run.npz, written by
tests/golden/make_golden_t42l20_run.py from the reference package (solid-body
basic state, elliptic heating at 0N 120E, plain damping, dt 1200 s, the
reference's default dynamics)."""

import types

import numpy as np
import pytest

from conftest import golden
from lbm_isca_gb300 import configs

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "fp32": 1e-5, "bf16x3": 1e-5, "bf16split": 1e-3}


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def _run(precision, ndays):
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(128, 64, sigm)
    heat = configs.elliptic_heating(128, 64, sigm)
    sp = Spectral(nlon=128, nlat=64, nmax=42, device="gb300")
    vg = VerticalGrid(sigm=sigm, device="gb300")
    m = LBM(bs, sp, vg, Config(ndays=ndays, precision=precision,
                               **configs.plain_damping(20)))
    sf = types.SimpleNamespace(t=heat, vor=None, div=None, ps=None)
    m.run(steady_forcing=sf, verbose=False)
    a, _ = m.stepper().spectral_state()
    return m, a


def _packed(x, M=43):
    x = x.detach().cpu().numpy()[0]
    mm, nn = np.nonzero(np.triu(np.ones((M, M), dtype=bool)))
    return x[mm, nn] if x.ndim == 2 else x[mm, nn, :]


@pytest.mark.parametrize("precision", ["fp64", "fp32", "bf16x3", "bf16split"])
@pytest.mark.parametrize("day", [10, 30])
def test_t42l20_run_matches_reference_trajectory(torch, precision, day):
    g = golden("t42l20_reference_run.npz")
    m, a = _run(precision, float(day))
    tol = TOL[precision]
    errs = {}
    for k in ("vor", "div", "t", "pi"):
        ref = g[f"day{day}_{k}"]
        got = _packed(a[k])
        errs[k] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    # q' stays zero (no moisture forcing, q-bar = 0): its absolute maximum
    errs["q_absmax"] = float(np.abs(_packed(a["q"])).max())
    ps = m.ga.ps.detach().cpu().numpy()
    errs["ps"] = float(np.linalg.norm(ps - g[f"day{day}_ps"]) /
                       np.linalg.norm(g[f"day{day}_ps"]))
    assert errs["q_absmax"] == 0.0, errs
    for k in ("vor", "div", "t", "pi", "ps"):
        assert errs[k] <= tol, (k, errs)
