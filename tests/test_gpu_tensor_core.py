"""The Legendre analysis and synthesis and the longitude analysis on the
tensor cores (tcgen05, bfloat16 split operands, FP32 accumulation in tensor
memory) against FP64 numpy restatements of the same contractions, next to
the FP32 FMA kernels they replace; and whole runs in the bf16 modes (their
default placement of the contractions) against the FP64 path."""

import ctypes as C

import numpy as np
import pytest

from oracle import lbm_oracle as orc
from lbm_isca_gb300 import configs

pytestmark = pytest.mark.gpu

CASES = {"T21L20": (64, 32, 21, 20, 5), "T42L20": (128, 64, 42, 20, 4),
         "T85L40": (256, 128, 85, 40, 2)}


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def _stepper(torch, case, precision):
    from lbm_isca_gb300 import Config
    from lbm_isca_gb300.ensemble import make_ensemble_model
    nlon, nlat, nmax, K, E = CASES[case]
    sigm = configs.equal_sigma_half_levels(K)
    bs = configs.solid_body_basic_state(nlon, nlat, sigm)
    m, _, _ = make_ensemble_model(bs, E, Config(precision=precision, **configs.plain_damping(K)),
                                  device="gb300", nlon=nlon, nlat=nlat, nmax=nmax, sigm=sigm)
    stp = m.stepper()
    # the kernel tests run every contraction on the tensor cores, whatever
    # the precision's default placement
    stp.tc_off = 0
    stp._desc = stp._oargs = None
    stp.set_timesteps([1200.0])
    return stp


def _oracle_analysis(tr, af, K):
    """tend [E][4][NS][K] of af [E][M][J][K][7] in FP64: for each m, rows n:
    vor = i m P.FV + H.FU, div = i m P.FU - H.FV + nn1a P.KE,
    T = P.T + H.XV, q = P.Q + H.YV (sums over every latitude)."""
    E, M = af.shape[:2]
    N = M - 1
    nn1a = -tr.lap
    out = []
    for e in range(E):
        rows = {f: [] for f in range(4)}
        for m in range(M):
            P, H = tr.P[m, m:, :], tr.H[m, m:, :]          # [n][j]
            x = af[e, m]                                    # [j][k][7]
            c = lambda T, f: T @ x[:, :, f]                 # noqa: E731  [n][k]
            rows[0].append(1j * m * c(P, 1) + c(H, 0))
            rows[1].append(1j * m * c(P, 0) - c(H, 1) + nn1a[m:, None] * c(P, 2))
            rows[2].append(c(P, 3) + c(H, 4))
            rows[3].append(c(P, 5) + c(H, 6))
        out.append(np.stack([np.concatenate(rows[f]) for f in range(4)]))
    return np.stack(out)


@pytest.mark.parametrize("case", list(CASES))
def test_analysis_kernel_vs_fp64(torch, case):
    from lbm_isca_gb300 import _lib
    from lbm_isca_gb300._lib import StepCtl, check, lib
    from lbm_isca_gb300.backend import stream_handle
    nlon, nlat, nmax, K, E = CASES[case]
    tr = orc.SphericalTransform(nlon, nlat, nmax)
    rng = np.random.default_rng(17)
    M, J = nmax + 1, nlat
    af = (rng.normal(size=(E, M, J, K, 7)) + 1j * rng.normal(size=(E, M, J, K, 7)))
    afs = (rng.normal(size=(E, M, J, 2)) + 1j * rng.normal(size=(E, M, J, 2)))
    ref = _oracle_analysis(tr, af, K)
    got, tends = {}, {}
    for prec in ("fp32", "bf16x3", "bf16split"):
        stp = _stepper(torch, case, prec)
        stp.af.copy_(torch.as_tensor(af, device="cuda").to(torch.complex64))
        stp.afs.copy_(torch.as_tensor(afs, device="cuda").to(torch.complex64))
        stp.tend.zero_()
        ctl = (StepCtl * 1)()
        ctl[0].dt, ctl[0].set, ctl[0].ps_mode, ctl[0].ra_mode = 1200.0, 0, 0, 1
        with torch.cuda.stream(stp.stream):
            check(lib().lbm_stepper_launch(C.byref(stp.desc()), ctl, 1,
                                           stream_handle(stp.stream)), "analysis")
        stp.stream.synchronize()
        assert int(stp.err.item()) == 0
        got[prec] = stp.tend.cpu().numpy().astype(np.complex128)
        tends[prec] = stp.tends.cpu().numpy()
    errs = {p: float(np.linalg.norm(g - ref) / np.linalg.norm(ref)) for p, g in got.items()}
    # the tensor-core surface part is the FMA kernel's own code
    assert np.array_equal(tends["bf16x3"], tends["fp32"])
    assert errs["fp32"] < 2e-6, errs
    assert errs["bf16x3"] < max(2e-6, 3 * errs["fp32"]), errs
    assert errs["bf16split"] < 1e-3, errs


def _oracle_longitude_analysis(g9, jfac, M):
    """af [E][M][J][K][7] and afs [E][M][J][2] of the grid rows g9
    [E][J][2 + 9K][I] in FP64: X = rfft / I of each row, then per level
    (rows gt xu g yu fu fv ke xv yv) FU = wd X(fu), FV = wd X(fv),
    KE = wg X(ke), T = wg X(gt) - wd i m X(xu), XV = wd X(xv),
    Q = wg X(g) - wd i m X(yu), YV = wd X(yv); surface rows wg X."""
    E, J, R, I = g9.shape
    K = (R - 2) // 9
    X = np.fft.rfft(g9, axis=-1)[..., :M] / I              # [E][J][R][M]
    wg, wd = jfac[0][None, :, None, None], jfac[1][None, :, None, None]
    lev = X[:, :, 2:].reshape(E, J, K, 9, M)               # [E][J][K][f][M]
    im = 1j * np.arange(M)
    f = lambda i: lev[:, :, :, i]                           # noqa: E731  [E][J][K][M]
    fields = [wd * f(4), wd * f(5), wg * f(6), wg * f(0) - wd * im * f(1),
              wd * f(7), wg * f(2) - wd * im * f(3), wd * f(8)]
    af = np.stack(fields, -1).transpose(0, 3, 1, 2, 4)     # [E][M][J][K][7]
    afs = (wg * X[:, :, :2]).transpose(0, 3, 1, 2)         # [E][M][J][2]
    return af, afs


@pytest.mark.parametrize("case", ["T21L20", "T42L20"])
def test_longitude_analysis_kernel_vs_fp64(torch, case):
    """Kernel 6 (grid rows -> af, afs): the FMA k_fdft in fp32 and the
    tensor-core k_fdft_tc in bf16x3 / bf16split against the FP64 rfft."""
    from lbm_isca_gb300._lib import StepCtl, check, lib
    from lbm_isca_gb300.backend import stream_handle
    nlon, nlat, nmax, K, E = CASES[case]
    M = nmax + 1
    rng = np.random.default_rng(23)
    g9 = rng.normal(size=(E, nlat, 2 + 9 * K, nlon)).astype(np.float32)
    got = {}
    ref = None
    for prec in ("fp32", "bf16x3", "bf16split"):
        stp = _stepper(torch, case, prec)
        if prec != "fp32":
            assert stp.tc_dft is not None
        if ref is None:
            jfac = stp.jfac.double().cpu().numpy()
            ref = _oracle_longitude_analysis(g9.astype(np.float64), jfac, M)
        stp.grid9.copy_(torch.as_tensor(g9, device="cuda"))
        stp.af.zero_()
        stp.afs.zero_()
        ctl = (StepCtl * 1)()
        ctl[0].dt, ctl[0].set, ctl[0].ps_mode, ctl[0].ra_mode = 1200.0, 0, 0, 1
        with torch.cuda.stream(stp.stream):
            check(lib().lbm_stepper_launch(C.byref(stp.desc()), ctl, 6,
                                           stream_handle(stp.stream)), "longitude analysis")
        stp.stream.synchronize()
        assert int(stp.err.item()) == 0
        got[prec] = (stp.af.cpu().numpy().astype(np.complex128),
                     stp.afs.cpu().numpy().astype(np.complex128))
    err = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))   # noqa: E731
    errs = {p: (err(a, ref[0]), err(b, ref[1])) for p, (a, b) in got.items()}
    e32 = max(errs["fp32"])
    assert e32 < 2e-6, errs
    assert max(errs["bf16x3"]) < max(2e-6, 3 * e32), errs
    assert max(errs["bf16split"]) < 1e-3, errs


def test_longitude_analysis_t85_stays_on_fma(torch):
    """nlon = 256 is past the tensor-core plan: no table, the FMA kernel runs."""
    stp = _stepper(torch, "T85L40", "bf16x3")
    assert stp.tc_dft is None


def _oracle_synthesis(tr, sa3, K):
    """sf [E][M][J][K][6] of the packed state sa3 [E][4][NS][K] in FP64:
    U = i m P il div - H il vor, V = i m P il vor + H il div, then P vor,
    P div, P T, P q (sums over n = m..N, every latitude)."""
    E = sa3.shape[0]
    M = tr.nmax + 1
    il = tr.invlap
    out = np.zeros((E, M, tr.nlat, K, 6), dtype=np.complex128)
    off = 0
    for m in range(M):
        nr = M - m
        sl = slice(off, off + nr)
        P, H, ilm = tr.P[m, m:, :], tr.H[m, m:, :], il[m:, None]
        for e in range(E):
            vo, dv, tt, qq = (sa3[e, f, sl] for f in range(4))       # [n][k]
            S = lambda T, x: T.T @ x                                   # noqa: E731 [j][k]
            out[e, m, :, :, 0] = 1j * m * S(P, ilm * dv) - S(H, ilm * vo)
            out[e, m, :, :, 1] = 1j * m * S(P, ilm * vo) + S(H, ilm * dv)
            out[e, m, :, :, 2] = S(P, vo)
            out[e, m, :, :, 3] = S(P, dv)
            out[e, m, :, :, 4] = S(P, tt)
            out[e, m, :, :, 5] = S(P, qq)
        off += nr
    return out


@pytest.mark.parametrize("case", list(CASES))
def test_synthesis_kernel_vs_fp64(torch, case):
    from lbm_isca_gb300._lib import StepCtl, check, lib
    from lbm_isca_gb300.backend import stream_handle
    nlon, nlat, nmax, K, E = CASES[case]
    tr = orc.SphericalTransform(nlon, nlat, nmax)
    M = nmax + 1
    NS = M * (M + 1) // 2
    rng = np.random.default_rng(23)
    sa3 = rng.normal(size=(E, 4, NS, K)) + 1j * rng.normal(size=(E, 4, NS, K))
    sa3[:, :, :M] = sa3[:, :, :M].real          # m = 0 rows are real
    sas = rng.normal(size=(E, 4, NS)) + 1j * rng.normal(size=(E, 4, NS))
    ref = _oracle_synthesis(tr, sa3, K)
    got, sfs = {}, {}
    for prec in ("fp32", "bf16x3", "bf16split"):
        stp = _stepper(torch, case, prec)
        stp.sa3.copy_(torch.as_tensor(sa3, device="cuda").to(torch.complex64))
        stp.sas.copy_(torch.as_tensor(sas, device="cuda").to(torch.complex64))
        stp.sf.zero_()
        ctl = (StepCtl * 1)()
        ctl[0].dt, ctl[0].set, ctl[0].ps_mode, ctl[0].ra_mode = 1200.0, 0, 0, 1
        with torch.cuda.stream(stp.stream):
            check(lib().lbm_stepper_launch(C.byref(stp.desc()), ctl, 3,
                                           stream_handle(stp.stream)), "synthesis")
        stp.stream.synchronize()
        assert int(stp.err.item()) == 0
        got[prec] = stp.sf.cpu().numpy().astype(np.complex128)
        sfs[prec] = stp.sfs.cpu().numpy()
    errs = {p: float(np.linalg.norm(g - ref) / np.linalg.norm(ref)) for p, g in got.items()}
    assert np.array_equal(sfs["bf16x3"], sfs["fp32"])
    assert errs["fp32"] < 2e-6, errs
    assert errs["bf16x3"] < max(2e-6, 3 * errs["fp32"]), errs
    assert errs["bf16split"] < 1e-3, errs


@pytest.mark.parametrize("precision,tol", [("bf16x3", 1e-5), ("bf16split", 1e-3)])
def test_bf16_ensemble_against_fp64_at_day10(torch, precision, tol):
    """Four seeded members at T42L20 for 10 days: every prognostic field
    within the mode's tolerance of the FP64 path (relative L2 over the packed
    spectral state)."""
    from lbm_isca_gb300 import Config
    from lbm_isca_gb300.ensemble import EnsembleForcing, make_ensemble_model
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(128, 64, sigm)
    heats, _ = configs.ensemble_heating(128, 64, sigm, 4, seed=1)
    out = {}
    for prec in ("fp64", precision):
        m, _, _ = make_ensemble_model(
            bs, 4, Config(ndays=10.0, precision=prec, **configs.plain_damping(20)),
            device="gb300", nlon=128, nlat=64, nmax=42, sigm=sigm)
        m.run(mjo_forcing=EnsembleForcing(heats, device="gb300"), verbose=False)
        a, _ = m.stepper().spectral_state()
        out[prec] = {k: v.cpu() for k, v in a.items()}
    for k in ("vor", "div", "t", "pi"):
        r, f = out["fp64"][k], out[precision][k]
        e = float(torch.linalg.norm(f - r) / torch.linalg.norm(r))
        assert e <= tol, (k, e)
    assert float(out[precision]["q"].abs().max()) == 0.0


@pytest.mark.parametrize("precision", ["bf16x3", "bf16split"])
def test_members_independent_of_ensemble_size(torch, precision):
    """Every contraction on the tensor cores: the first two members of a
    32-member ensemble (13 units per persistent CTA, so the operand rings and
    the two accumulator sets cycle many times) step bit for bit like a
    2-member ensemble with the same heatings, over 24 steps."""
    from lbm_isca_gb300 import Config
    from lbm_isca_gb300.ensemble import make_ensemble_model
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(128, 64, sigm)
    heats, _ = configs.ensemble_heating(128, 64, sigm, 32, seed=3)
    got = {}
    for E in (2, 32):
        m, _, _ = make_ensemble_model(
            bs, E, Config(ndays=1.0, precision=precision, tc_off=0, **configs.plain_damping(20)),
            device="gb300", nlon=128, nlat=64, nmax=42, sigm=sigm)
        stp = m.stepper()
        sched = m._schedule(24)
        stp.set_timesteps(sorted({dt for dt, _ in sched}))
        stp.set_forcing(frc_t=m._spec_forcing(torch.as_tensor(heats[:E], device="cuda"), True),
                        per_member=True)
        stp.load_zero()
        stp.run(sched, use_graph=True)
        torch.cuda.synchronize()
        assert stp.check_finite()
        got[E] = (stp.sa3[:2].clone(), stp.sas[:2].clone(), stp.psa[:2].clone())
    for a, b in zip(got[2], got[32]):
        assert torch.equal(a, b)
