"""lbm_stepper_run_noalloc (the stepper whose intermediates live in the
library's static scratch area) against lbm_stepper_prime + lbm_stepper_run
on caller buffers, through the C ABI, over two calls in a row.

The file is collected last, so that in a full `-m gpu` run it also shows the
entry point working after every other test has used the device; run alone it
covers the first-call set-up in a fresh process."""

import ctypes as C

import numpy as np
import pytest

from lbm_isca_gb300 import configs

pytestmark = pytest.mark.gpu

DT = 1200.0            # T21: 72 steps a day
TOL = {"fp64": 1e-12, "fp32": 1e-6}
SCRATCH = ("sf", "sfs", "af", "afs", "tend", "tends", "grid6", "grid9")
STATE = ("sa3", "sas", "sb3", "psa", "psb")


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _stepper(torch, precision, nmem):
    """T21L20 ensemble stepper with a seeded random state and a T forcing."""
    from lbm_isca_gb300 import Config
    from lbm_isca_gb300.ensemble import make_ensemble_model
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    m, _, _ = make_ensemble_model(bs, nmem, Config(ndays=1.0, precision=precision,
                                                   **configs.plain_damping(20)),
                                  device="gb300", nlon=64, nlat=32, nmax=21, sigm=sigm)
    stp = m.stepper()
    stp.set_timesteps([DT])
    g = torch.Generator().manual_seed(7)
    M, K, E = stp.M, stp.K, nmem

    def spec(scale, k=True):
        shape = (E, M, M, K) if k else (E, M, M)
        z = torch.randn(shape + (2,), generator=g, dtype=torch.float64) * scale
        return torch.view_as_complex(z).cuda()

    scales = {"vor": 1e-6, "div": 1e-6, "t": 0.5, "q": 1e-4}
    a = {k: spec(s) for k, s in scales.items()}
    b = {k: spec(s) for k, s in scales.items()}
    a["pi"] = spec(1e-3, k=False)
    ps = lambda: (torch.randn((E, stp.J, stp.I), generator=g, dtype=torch.float64)  # noqa: E731
                  * 100.0).cuda()
    stp.set_forcing(frc_t=spec(1e-5)[0])
    stp.load(a, b, ps(), ps())
    torch.cuda.synchronize()
    return stp


def _ctl(steps):
    from lbm_isca_gb300._lib import StepCtl
    arr = (StepCtl * len(steps))()
    for i, (psm, ra) in enumerate(steps):
        arr[i].dt, arr[i].set, arr[i].ps_mode, arr[i].ra_mode = DT, 0, psm, ra
    return arr


# first call: continue from a freshly loaded state (ps up to date), then the
# filtered leapfrog; second call: filtered leapfrog throughout
CALLS = (_ctl([(0, 1), (2, 1), (2, 1)]), _ctl([(2, 1), (2, 1), (2, 1)]))


def _state(stp):
    return [getattr(stp, n).clone() for n in STATE]


def _relerr(got, ref):
    got, ref = got.cpu().numpy(), ref.cpu().numpy()
    den = np.max(np.abs(ref))
    return float(np.max(np.abs(got - ref)) / (den if den > 0 else 1.0))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_matches_caller_buffer_stepper(torch, precision):
    from lbm_isca_gb300._lib import LBM_OK, StepperDesc, lib
    L = lib()
    stp = _stepper(torch, precision, nmem=2)
    s = C.c_void_p(stp.stream.cuda_stream)
    d = stp.desc()
    init = _state(stp)

    ref = []
    for ctl in CALLS:
        assert L.lbm_stepper_run(C.byref(d), ctl, len(ctl), s) == LBM_OK
        torch.cuda.synchronize()
        ref.append(_state(stp))
    assert int(stp.err.item()) == 0

    for n, x in zip(STATE, init):
        getattr(stp, n).copy_(x)
    # the caller passes no intermediate buffers
    dn = StepperDesc.from_buffer_copy(d)
    for n in SCRATCH:
        setattr(dn, n, None)
    for call, ctl in enumerate(CALLS):
        assert L.lbm_stepper_run_noalloc(C.byref(dn), ctl, len(ctl), s) == LBM_OK
        torch.cuda.synchronize()
        got = _state(stp)
        for n, x, r in zip(STATE, got, ref[call]):
            assert bool(torch.isfinite(torch.view_as_real(x) if x.is_complex() else x).all())
            e = _relerr(x, r)
            assert e <= TOL[precision], (precision, call, n, e)
    assert int(stp.err.item()) == 0


def test_noalloc_rejects_a_case_beyond_the_scratch_area(torch):
    from lbm_isca_gb300._lib import (LBM_ERR_SCRATCH, LBM_NOALLOC_SCRATCH_BYTES, StepperDesc,
                                     lib)
    stp = _stepper(torch, "fp32", nmem=2)
    dn = StepperDesc.from_buffer_copy(stp.desc())
    # 64 members at T21L20 in FP32 need about 100 MiB of intermediates
    dn.nmem = 64
    M, J, K = stp.M, stp.J, stp.K
    need = 64 * (M * J * (13 * K + 7) + stp.NS * (4 * K + 2)) * 8
    assert need > LBM_NOALLOC_SCRATCH_BYTES
    before = _state(stp)
    ctl = CALLS[0]
    assert lib().lbm_stepper_run_noalloc(C.byref(dn), ctl, len(ctl),
                                         C.c_void_p(stp.stream.cuda_stream)) == LBM_ERR_SCRATCH
    torch.cuda.synchronize()
    for x, y in zip(before, _state(stp)):
        assert torch.equal(x, y)
