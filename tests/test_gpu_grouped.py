"""Uneven batching: members of several truncations and level counts stepped
together in one CUDA graph per stretch of steady steps (one branch per
group) equal each group run alone through LBM.run, bit for bit."""

import numpy as np
import pytest

from lbm_isca_gb300 import configs

pytestmark = pytest.mark.gpu

GROUPS = [(64, 32, 21, 20, 6), (128, 64, 42, 20, 4), (256, 128, 85, 40, 2)]


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.parametrize("precision", ["fp64", "bf16x3"])
def test_grouped_ensemble_matches_groups_run_alone(torch, precision):
    from lbm_isca_gb300 import Config, autotune
    from lbm_isca_gb300.ensemble import EnsembleForcing, make_ensemble_model
    from lbm_isca_gb300.grouped import GroupedEnsemble
    nsteps = 30
    sig = {K: configs.equal_sigma_half_levels(K) for K in (20, 40)}
    heats = configs.grouped_heating([(nlon, nlat, sig[K], E)
                                     for nlon, nlat, _, K, E in GROUPS], seed=4)
    groups = []
    for (nlon, nlat, nmax, K, E), h in zip(GROUPS, heats):
        groups.append(dict(nlon=nlon, nlat=nlat, nmax=nmax, sigm=sig[K], heats=h,
                           basic_state=configs.solid_body_basic_state(nlon, nlat, sig[K]),
                           config=dict(configs.plain_damping(K), strictly_linear=True)))
    ge = GroupedEnsemble(groups, precision=precision, tune=True)
    ge.run(nsteps)
    assert ge.check_finite()
    together = ge.spectral_states()
    for grp, g, ref_state in zip(ge.groups, groups, together):
        m, _, _ = make_ensemble_model(
            g["basic_state"], len(g["heats"]),
            Config(ndays=nsteps / 72.0, precision=precision, **g["config"]),
            device="gb300", nlon=g["nlon"], nlat=g["nlat"], nmax=g["nmax"], sigm=g["sigm"])
        stp = m.stepper()
        if grp["tile"] is not None:
            autotune._apply(stp, grp["tile"]["tc_off"], grp["tile"]["tc_g"])
        m.run(mjo_forcing=EnsembleForcing(g["heats"], device="gb300"), verbose=False)
        alone, _ = stp.spectral_state()
        for k in ("vor", "div", "t", "pi", "q"):
            assert torch.equal(alone[k], ref_state[k]), (g["nmax"], k)
