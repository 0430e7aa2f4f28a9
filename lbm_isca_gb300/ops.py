"""The C ABI of include/lbm_gb300.h as PyTorch operators, ``torch.ops.lbm_gb300.*``.

Each operator is a thin wrapper over one ``extern "C"`` entry point of the
library (loaded through ``_lib``): it checks dtypes, allocates its outputs
with torch, launches on the current CUDA stream and raises on a nonzero
status.  The operators are registered for CUDA tensors only (there is no CPU
path), and each has a fake (meta) implementation that gives the output
shapes without running anything, so they compose with torch's tracing and
graph-capture machinery.  The package's classes call these operators:
``Spectral`` (transforms, set-up tables), ``Dynamics`` (grid-point
tendency), ``Integrator`` (semi-implicit step), ``SemiImplicit`` and
``VerticalDiffusion`` (matrices and inverses), the adjoint's ``TimeStep``
and the fused ``EnsembleStepper`` (per-step runs, priming, column sums, the
final ps update, the history sums).

Conventions of the list arguments:
* a zero-element tensor in a ``Tensor[]`` list stands for a NULL pointer;
* ``Tensor?[]`` lists take None for NULL;
* integer / float lists carry the sizes and constants of the C structs in
  the order the header declares them.

Where the reference selects its array module (backend.py:53-77), the
``"gb300"`` device value selects these operators.
"""

from __future__ import annotations

import ctypes as C
from typing import List, Optional

import torch
from torch import Tensor

from . import _lib
from ._lib import (ImplicitAdjArgs, ImplicitArgs, StepCtl, StepperDesc, TendAdjArgs,
                   TendGridArgs, check, lib)

NS_ = "lbm_gb300"


def _prec(t):
    if t.dtype in (torch.float64, torch.complex128):
        return _lib.LBM_F64
    if t.dtype in (torch.float32, torch.complex64):
        return _lib.LBM_F32
    raise TypeError(f"lbm_gb300: unsupported dtype {t.dtype}")


def _same(prec, *ts):
    """Every given tensor in the precision `prec` (real or complex)."""
    for t in ts:
        if t is not None and t.numel() and _prec(t) != prec:
            raise TypeError(f"lbm_gb300: mixed precisions ({t.dtype} in a "
                            f"{'FP64' if prec == _lib.LBM_F64 else 'FP32'} call)")


def _cplx(prec):
    return torch.complex128 if prec == _lib.LBM_F64 else torch.complex64


def _real(prec):
    return torch.float64 if prec == _lib.LBM_F64 else torch.float32


def _p(t):
    """Device pointer of an optional tensor (None or zero elements -> NULL)."""
    if t is None or t.numel() == 0:
        return None
    return C.c_void_p(t.data_ptr())


def _st():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class _Keep:
    """Inputs as the C ABI wants them: contiguous, copied if they are not.
    The copies are held here until the library call has queued its launch
    (stream order then keeps their memory from being reused before the
    kernel has read them); a copy dropped earlier could be handed to the next
    copy of the same call and overwritten before the kernel runs."""

    def __init__(self):
        self.held = []

    def __call__(self, t):
        if t is None:
            return None
        c = t.contiguous()
        self.held.append(c)
        return c


def _w(t):
    """A tensor the operator writes in place: must already be contiguous."""
    if t is not None and t.numel() and not t.is_contiguous():
        raise ValueError("lbm_gb300: tensors written in place must be contiguous")
    return t


# =============================================================================
# set-up (FP64): spectral.py:49-154, integrator.py:130-163, 226
# =============================================================================
@torch.library.custom_op(f"{NS_}::gauss_legendre", mutates_args=(), device_types="cuda")
def gauss_legendre(like: Tensor, nlat: int) -> List[Tensor]:
    """(mu, gw) of `nlat` Gauss-Legendre latitudes, north first, sum gw = 1
    (lbm_gauss_legendre).  `like` names the device."""
    mu = torch.empty(nlat, device=like.device, dtype=torch.float64)
    gw = torch.empty_like(mu)
    check(lib().lbm_gauss_legendre(nlat, _p(mu), _p(gw), _st()), "lbm_gauss_legendre")
    return [mu, gw]


@gauss_legendre.register_fake
def _(like, nlat):
    return [like.new_empty(nlat, dtype=torch.float64), like.new_empty(nlat, dtype=torch.float64)]


@torch.library.custom_op(f"{NS_}::legendre_tables", mutates_args=(), device_types="cuda")
def legendre_tables(mu: Tensor, nmax: int) -> List[Tensor]:
    """(P, H) [M][M][nlat] (lbm_legendre_tables)."""
    keep = _Keep()
    M, J = nmax + 1, mu.shape[0]
    P = torch.empty((M, M, J), device=mu.device, dtype=torch.float64)
    H = torch.empty_like(P)
    check(lib().lbm_legendre_tables(nmax, J, _p(keep(mu)), _p(P), _p(H), _st()),
          "lbm_legendre_tables")
    return [P, H]


@legendre_tables.register_fake
def _(mu, nmax):
    M, J = nmax + 1, mu.shape[0]
    return [mu.new_empty((M, M, J)), mu.new_empty((M, M, J))]


@torch.library.custom_op(f"{NS_}::fft_twiddles", mutates_args=(), device_types="cuda")
def fft_twiddles(like: Tensor, nlon: int) -> Tensor:
    """exp(-2 pi i p / nlon), complex FP64 [nlon] (lbm_fft_twiddles)."""
    tw = torch.empty(nlon, device=like.device, dtype=torch.complex128)
    check(lib().lbm_fft_twiddles(nlon, _p(tw), _st()), "lbm_fft_twiddles")
    return tw


@fft_twiddles.register_fake
def _(like, nlon):
    return like.new_empty(nlon, dtype=torch.complex128)


@torch.library.custom_op(f"{NS_}::gravity_wave_matrices", mutates_args=(),
                         device_types="cuda")
def gravity_wave_matrices(lap: Tensor, ktt: Tensor, kd: Tensor, whmtx: Tensor, gcmtx: Tensor,
                          dt: float) -> Tensor:
    """M(n) [M][K][K] of the semi-implicit scheme (lbm_gravity_wave_matrices)."""
    keep = _Keep()
    M, K = ktt.shape
    mats = torch.empty((M, K, K), device=lap.device, dtype=torch.float64)
    check(lib().lbm_gravity_wave_matrices(M - 1, K, float(dt), _p(keep(lap)), _p(keep(ktt)),
                                          _p(keep(kd)), _p(keep(whmtx)), _p(keep(gcmtx)), _p(mats),
                                          _st()), "lbm_gravity_wave_matrices")
    return mats


@gravity_wave_matrices.register_fake
def _(lap, ktt, kd, whmtx, gcmtx, dt):
    M, K = ktt.shape
    return lap.new_empty((M, K, K))


@torch.library.custom_op(f"{NS_}::batched_inverse", mutates_args=(), device_types="cuda")
def batched_inverse(a: Tensor) -> List[Tensor]:
    """(a^-1, info) of a [batch][n][n] FP64 stack (lbm_batched_inverse); info
    is 0 or 1 + the column of a zero pivot."""
    keep = _Keep()
    B, n, _ = a.shape
    out = torch.empty_like(a)
    info = torch.empty(B, device=a.device, dtype=torch.int32)
    check(lib().lbm_batched_inverse(B, n, _p(keep(a)), _p(out), _p(info), _st()),
          "lbm_batched_inverse")
    return [out, info]


@batched_inverse.register_fake
def _(a):
    return [torch.empty_like(a), a.new_empty(a.shape[0], dtype=torch.int32)]


# =============================================================================
# spectral transforms on the reference layouts (spectral.py:159-276)
# =============================================================================
@torch.library.custom_op(f"{NS_}::fourier_forward", mutates_args=(), device_types="cuda")
def fourier_forward(grid: Tensor, jscale: Optional[Tensor], tw: Tensor, nmax: int) -> Tensor:
    """four[B][M][J][C] = jscale[j] / nlon rfft(grid[B][J][I][C]) for m <= nmax
    (lbm_fourier_forward; Spectral._fft_fwd, spectral.py:159-164)."""
    keep = _Keep()
    prec = _prec(grid)
    _same(prec, jscale, tw)
    B, J, I, Cn = grid.shape
    four = torch.empty((B, nmax + 1, J, Cn), device=grid.device, dtype=_cplx(prec))
    check(lib().lbm_fourier_forward(prec, B, J, I, Cn, nmax, _p(keep(grid)), _p(keep(jscale)),
                                    _p(keep(tw)), _p(four), _st()), "lbm_fourier_forward")
    return four


@fourier_forward.register_fake
def _(grid, jscale, tw, nmax):
    B, J, I, Cn = grid.shape
    return grid.new_empty((B, nmax + 1, J, Cn), dtype=_cplx(_prec(grid)))


@torch.library.custom_op(f"{NS_}::fourier_inverse", mutates_args=(), device_types="cuda")
def fourier_inverse(four: Tensor, jscale: Optional[Tensor], tw: Tensor, nlon: int) -> Tensor:
    """grid[B][J][nlon][C] = jscale[j] irfft(nlon four) (lbm_fourier_inverse;
    Spectral._fft_inv, spectral.py:166-172)."""
    keep = _Keep()
    prec = _prec(four)
    _same(prec, jscale, tw)
    B, M, J, Cn = four.shape
    g = torch.empty((B, J, nlon, Cn), device=four.device, dtype=_real(prec))
    check(lib().lbm_fourier_inverse(prec, B, J, nlon, Cn, M - 1, _p(keep(four)), _p(keep(jscale)),
                                    _p(keep(tw)), _p(g), _st()), "lbm_fourier_inverse")
    return g


@fourier_inverse.register_fake
def _(four, jscale, tw, nlon):
    B, M, J, Cn = four.shape
    return four.new_empty((B, J, nlon, Cn), dtype=_real(_prec(four)))


@torch.library.custom_op(f"{NS_}::legendre_analysis", mutates_args=(), device_types="cuda")
def legendre_analysis(fa: Tensor, ta: Tensor, ima: int, fb: Optional[Tensor],
                      tb: Optional[Tensor], imb: int, sb: float,
                      nfac: Optional[Tensor]) -> Tensor:
    """spec[B][M][M][C] from Fourier fields [B][M][J][C] and tables [M][M][J]
    (lbm_legendre_analysis; the matmuls of spectral.py:190, 242-243)."""
    keep = _Keep()
    prec = _prec(fa)
    _same(prec, ta, fb, tb, nfac)
    B, M, J, Cn = fa.shape
    spec = torch.empty((B, M, M, Cn), device=fa.device, dtype=_cplx(prec))
    check(lib().lbm_legendre_analysis(prec, B, M - 1, J, Cn, _p(keep(fa)), _p(keep(ta)), ima,
                                      _p(keep(fb)), _p(keep(tb)), imb, float(sb), _p(keep(nfac)), 0,
                                      _p(spec), _st()), "lbm_legendre_analysis")
    return spec


@legendre_analysis.register_fake
def _(fa, ta, ima, fb, tb, imb, sb, nfac):
    B, M, J, Cn = fa.shape
    return fa.new_empty((B, M, M, Cn))


@torch.library.custom_op(f"{NS_}::legendre_synthesis", mutates_args=(), device_types="cuda")
def legendre_synthesis(sa: Tensor, ta: Tensor, ima: int, na: Optional[Tensor],
                       sbp: Optional[Tensor], tb: Optional[Tensor], imb: int,
                       nb: Optional[Tensor], sb: float) -> Tensor:
    """four[B][M][J][C] from spectral fields [B][M][M][C] and tables [M][M][J]
    (lbm_legendre_synthesis; spectral.py:196, 220-221, 271-272)."""
    keep = _Keep()
    prec = _prec(sa)
    _same(prec, ta, na, sbp, tb, nb)
    B, M, _, Cn = sa.shape
    J = ta.shape[-1]
    four = torch.empty((B, M, J, Cn), device=sa.device, dtype=_cplx(prec))
    check(lib().lbm_legendre_synthesis(prec, B, M - 1, J, Cn, _p(keep(sa)), _p(keep(ta)), ima,
                                       _p(keep(na)), _p(keep(sbp)), _p(keep(tb)), imb, _p(keep(nb)),
                                       float(sb), _p(four), _st()), "lbm_legendre_synthesis")
    return four


@legendre_synthesis.register_fake
def _(sa, ta, ima, na, sbp, tb, imb, nb, sb):
    B, M, _, Cn = sa.shape
    return sa.new_empty((B, M, ta.shape[-1], Cn))


# =============================================================================
# grid-point tendency, semi-implicit step and their adjoints
# =============================================================================
TEND_INPUTS = ("dsig", "sigm", "alpha", "w3", "wP", "cpg", "sig", "ww", "tmtx", "tref",
               "ub", "vb", "tb", "qb", "tvb", "absvor", "divb", "x5b", "sdotb", "pixb", "piyb",
               "psb", "u", "v", "t", "q", "vor", "div", "pix", "piy", "ps", "frc_t", "frc_ps",
               "frc_q", "lin_u", "lin_v")
TEND_OUTPUTS = ("fu", "fv", "ke", "gt", "xu", "xv", "g", "yu", "yv", "gt_pi", "omega", "sdot")


def _tend_shapes(ins, kmax):
    u = ins[TEND_INPUTS.index("u")]
    s3 = tuple(u.shape)
    s2 = s3[:-1]
    return s3, s2, s2 + (kmax + 1,)


@torch.library.custom_op(f"{NS_}::tendency_grid", mutates_args=(), device_types="cuda")
def tendency_grid(ins: List[Optional[Tensor]], nmem: int, nlat: int, nlon: int, kmax: int,
                  strictly_linear: int, consts: List[float], frc_strides: List[int],
                  want_omega: bool) -> List[Tensor]:
    """Grid-point part of Dynamics.tendencies (dynamics.py:176-267) in one
    launch (lbm_tendency_grid).  `ins` in TEND_INPUTS order; consts = (kappa,
    epsvt, rair); frc_strides = member strides of frc_t, frc_ps, frc_q.
    Returns the TEND_OUTPUTS (omega has zero elements unless want_omega)."""
    keep = _Keep()
    u = ins[TEND_INPUTS.index("u")]
    _same(_prec(u), *ins)
    s3, s2, ssd = _tend_shapes(ins, kmax)
    f = dict(device=u.device, dtype=u.dtype)
    outs = [torch.empty(s3, **f) for _ in range(9)] + [torch.empty(s2, **f)]
    outs.append(torch.empty(s3, **f) if want_omega else torch.empty(0, **f))
    outs.append(torch.empty(ssd, **f))
    a = TendGridArgs()
    a.nmem, a.nlat, a.nlon, a.kmax = nmem, nlat, nlon, kmax
    a.strictly_linear = int(strictly_linear)
    a.kappa, a.epsvt, a.rair = (float(x) for x in consts)
    for name, t in zip(TEND_INPUTS, ins):
        setattr(a, name, _p(keep(t)))
    a.frc_t_stride, a.frc_ps_stride, a.frc_q_stride = (int(x) for x in frc_strides)
    for name, t in zip(TEND_OUTPUTS, outs):
        setattr(a, name, _p(t))
    check(lib().lbm_tendency_grid(_prec(u), a, _st()), "lbm_tendency_grid")
    return outs


@tendency_grid.register_fake
def _(ins, nmem, nlat, nlon, kmax, strictly_linear, consts, frc_strides, want_omega):
    u = ins[TEND_INPUTS.index("u")]
    s3, s2, ssd = _tend_shapes(ins, kmax)
    outs = [u.new_empty(s3) for _ in range(9)] + [u.new_empty(s2)]
    outs.append(u.new_empty(s3) if want_omega else u.new_empty(0))
    outs.append(u.new_empty(ssd))
    return outs


IMPL_OPS = ("lap", "kv", "kd", "ktt", "kq", "ww", "tmtx", "gg", "dsig", "minv", "vd_vor",
            "vd_div", "vd_t", "vd_q")
FIELDS5 = ("vor", "div", "t", "pi", "q")


@torch.library.custom_op(f"{NS_}::implicit_step", mutates_args=(), device_types="cuda")
def implicit_step(ops: List[Optional[Tensor]], prev: List[Tensor], tend: List[Tensor],
                  nmem: int, nmax: int, kmax: int, dt: float) -> List[Tensor]:
    """Integrator.step (integrator.py:264-315) on the rectangle layout
    (lbm_implicit_step): operators in IMPL_OPS order, previous level and
    explicit tendencies as (vor, div, t, pi, q); returns the new level."""
    keep = _Keep()
    _same(_prec(prev[0]), *ops, *prev, *tend)
    out = [torch.empty_like(x) for x in prev]
    a = ImplicitArgs()
    a.nmem, a.nmax, a.kmax, a.dt = nmem, nmax, kmax, float(dt)
    for name, t in zip(IMPL_OPS, ops):
        setattr(a, name, _p(keep(t)))
    for pre, lst in (("p_", prev), ("w_", tend), ("n_", out)):
        for k, t in zip(FIELDS5, lst):
            setattr(a, pre + k, _p(keep(t)))
    check(lib().lbm_implicit_step(_prec(prev[0]), a, _st()), "lbm_implicit_step")
    return out


@implicit_step.register_fake
def _(ops, prev, tend, nmem, nmax, kmax, dt):
    return [torch.empty_like(x) for x in prev]


TADJ_INPUTS = ("dsig", "sigm", "alpha", "w3", "wP", "cpg", "ww", "tmtx", "tref", "ub", "vb",
               "tb", "qb", "tvb", "absvor", "divb", "x5b", "sdotb", "pixb", "piyb", "u0", "v0",
               "a_fu", "a_fv", "a_ke", "a_gt", "a_xu", "a_xv", "a_g", "a_yu", "a_yv", "a_gt_pi")
TADJ_OUTPUTS = ("a_u", "a_v", "a_t", "a_q", "a_vor", "a_div", "a_pix", "a_piy")


@torch.library.custom_op(f"{NS_}::tendency_grid_adjoint", mutates_args=(),
                         device_types="cuda")
def tendency_grid_adjoint(ins: List[Optional[Tensor]], nmem: int, nlat: int, nlon: int,
                          kmax: int, consts: List[float]) -> List[Tensor]:
    """Transpose of the linearised grid-point tendency
    (lbm_tendency_grid_adjoint; no reference counterpart).  `ins` in
    TADJ_INPUTS order; returns TADJ_OUTPUTS."""
    keep = _Keep()
    afu = ins[TADJ_INPUTS.index("a_fu")]
    _same(_prec(afu), *ins)
    s3 = tuple(afu.shape)
    outs = [torch.empty(s3, device=afu.device, dtype=afu.dtype) for _ in range(6)]
    outs += [torch.empty(s3[:-1], device=afu.device, dtype=afu.dtype) for _ in range(2)]
    a = TendAdjArgs()
    a.nmem, a.nlat, a.nlon, a.kmax = nmem, nlat, nlon, kmax
    a.kappa, a.epsvt, a.rair = (float(x) for x in consts)
    for name, t in zip(TADJ_INPUTS, ins):
        setattr(a, name, _p(keep(t)))
    for name, t in zip(TADJ_OUTPUTS, outs):
        setattr(a, name, _p(t))
    check(lib().lbm_tendency_grid_adjoint(_prec(afu), a, _st()), "lbm_tendency_grid_adjoint")
    return outs


@tendency_grid_adjoint.register_fake
def _(ins, nmem, nlat, nlon, kmax, consts):
    afu = ins[TADJ_INPUTS.index("a_fu")]
    s3 = tuple(afu.shape)
    return [afu.new_empty(s3) for _ in range(6)] + [afu.new_empty(s3[:-1]) for _ in range(2)]


@torch.library.custom_op(f"{NS_}::implicit_step_adjoint", mutates_args=(),
                         device_types="cuda")
def implicit_step_adjoint(ops: List[Optional[Tensor]], an: List[Tensor], nmem: int, nmax: int,
                          kmax: int, dt: float) -> List[Tensor]:
    """Transpose of Integrator.step (lbm_implicit_step_adjoint): adjoint of
    the new level -> adjoints of the previous level and of the tendencies,
    (vor, div, t, pi, q) each."""
    keep = _Keep()
    _same(_prec(an[0]), *ops, *an)
    ap = [torch.empty_like(x) for x in an]
    aw = [torch.empty_like(x) for x in an]
    a = ImplicitAdjArgs()
    a.nmem, a.nmax, a.kmax, a.dt = nmem, nmax, kmax, float(dt)
    for name, t in zip(IMPL_OPS, ops):
        setattr(a, name, _p(keep(t)))
    for pre, lst in (("an_", an), ("ap_", ap), ("aw_", aw)):
        for k, t in zip(FIELDS5, lst):
            setattr(a, pre + k, _p(keep(t)))
    check(lib().lbm_implicit_step_adjoint(_prec(an[0]), a, _st()),
          "lbm_implicit_step_adjoint")
    return ap + aw


@implicit_step_adjoint.register_fake
def _(ops, an, nmem, nmax, kmax, dt):
    return [torch.empty_like(x) for x in an] + [torch.empty_like(x) for x in an]


# =============================================================================
# fused ensemble stepper (lbm_stepper_*)
# =============================================================================
STEP_STATE = ("sa3", "sas", "sb3", "psa", "psb", "err", "err_member")
STEP_WORK = ("sf", "sfs", "af", "afs", "tend", "tends", "grid6", "grid9")
STEP_OPS = ("symp", "symh", "tw", "jfac", "vert", "b3", "bsd", "b2", "lap", "invlap", "nn1a",
            "kv", "kd", "ktt", "kq", "ww", "tmtx", "minv", "vdiff", "frc3", "frcs", "dft",
            "tc_anal", "tc_synth", "tc_dft")
STEP_DIMS = ("prec", "nmem", "nlat", "nlon", "nmax", "kmax", "nsets", "strictly_linear",
             "vd_on0", "vd_on1", "vd_on2", "vd_on3", "frc_shared", "legendre", "tc_off", "tc_g")

_DESC_CACHE = {}


def _desc(state, work, ops, dims, consts):
    """lbm_stepper_desc of the operator arguments, cached by its pointers."""
    tens = list(state) + list(work) + list(ops)
    for t in list(state) + list(work):
        _w(t)
    key = (tuple(0 if t is None or t.numel() == 0 else t.data_ptr() for t in tens),
           tuple(dims), tuple(consts))
    d = _DESC_CACHE.get(key)
    if d is not None:
        return d
    d = StepperDesc()
    (d.prec, d.nmem, d.nlat, d.nlon, d.nmax, d.kmax, d.nsets, d.strictly_linear) = dims[:8]
    for i in range(4):
        d.vd_on[i] = dims[8 + i]
    d.frc_shared = dims[12]
    d.legendre, d.tc_off, d.tc_g = dims[13], dims[14], dims[15]
    d.kappa, d.epsvt, d.robert = (float(x) for x in consts)
    for name, t in zip(STEP_OPS + STEP_WORK, list(ops) + list(work)):
        setattr(d, name, _p(t))
    d.sa3, d.sas, d.sb3, d.psa, d.psb = (_p(t) for t in state[:5])
    for name, t in (("err", state[5]), ("err_member", state[6])):
        setattr(d, name, None if t.numel() == 0 else
                C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_int)))
    if len(_DESC_CACHE) > 64:
        _DESC_CACHE.clear()
    _DESC_CACHE[key] = d
    return d


def _ctl(dt, sets, ps_mode, ra_mode):
    arr = (StepCtl * len(dt))()
    for i in range(len(dt)):
        arr[i].dt = float(dt[i])
        arr[i].set = int(sets[i])
        arr[i].ps_mode = int(ps_mode[i])
        arr[i].ra_mode = int(ra_mode[i])
    return arr


@torch.library.custom_op(f"{NS_}::stepper_run", mutates_args=("state", "work"),
                         device_types="cuda")
def stepper_run(state: List[Tensor], work: List[Tensor], ops: List[Tensor], dims: List[int],
                consts: List[float], dt: List[float], sets: List[int], ps_mode: List[int],
                ra_mode: List[int]) -> None:
    """len(dt) steps of the fused stepper (lbm_stepper_run; the loop body of
    LBM.run, model.py:213-247): state in STEP_STATE order (updated in place),
    intermediates in STEP_WORK order, operators in STEP_OPS order, sizes in
    STEP_DIMS order, consts = (kappa, epsvt, robert), one (dt, operator set,
    ps_mode, ra_mode) per step as lbm_step_ctl describes."""
    d = _desc(state, work, ops, dims, consts)
    ctl = _ctl(dt, sets, ps_mode, ra_mode)
    check(lib().lbm_stepper_run(C.byref(d), ctl, len(dt), _st()), "lbm_stepper_run")


@stepper_run.register_fake
def _(state, work, ops, dims, consts, dt, sets, ps_mode, ra_mode):
    return None


@torch.library.custom_op(f"{NS_}::stepper_prime", mutates_args=("state", "work"),
                         device_types="cuda")
def stepper_prime(state: List[Tensor], work: List[Tensor], ops: List[Tensor], dims: List[int],
                  consts: List[float]) -> None:
    """Synthesis of the current level into the intermediates
    (lbm_stepper_prime)."""
    d = _desc(state, work, ops, dims, consts)
    check(lib().lbm_stepper_prime(C.byref(d), _st()), "lbm_stepper_prime")


@stepper_prime.register_fake
def _(state, work, ops, dims, consts):
    return None


@torch.library.custom_op(f"{NS_}::stepper_colsum", mutates_args=("state", "work"),
                         device_types="cuda")
def stepper_colsum(state: List[Tensor], work: List[Tensor], ops: List[Tensor],
                   dims: List[int], consts: List[float]) -> None:
    """Column sums of a freshly loaded current level (lbm_stepper_colsum)."""
    d = _desc(state, work, ops, dims, consts)
    check(lib().lbm_stepper_colsum(C.byref(d), _st()), "lbm_stepper_colsum")


@stepper_colsum.register_fake
def _(state, work, ops, dims, consts):
    return None


@torch.library.custom_op(f"{NS_}::stepper_flush", mutates_args=("state", "work"),
                         device_types="cuda")
def stepper_flush(state: List[Tensor], work: List[Tensor], ops: List[Tensor], dims: List[int],
                  consts: List[float], ps_mode: int) -> None:
    """Apply the pending grid-ps update (lbm_stepper_flush)."""
    d = _desc(state, work, ops, dims, consts)
    check(lib().lbm_stepper_flush(C.byref(d), int(ps_mode), _st()), "lbm_stepper_flush")


@stepper_flush.register_fake
def _(state, work, ops, dims, consts, ps_mode):
    return None


@torch.library.custom_op(f"{NS_}::history_accumulate", mutates_args=("prev", "acc"),
                         device_types="cuda")
def history_accumulate(cur: Tensor, prev: Tensor, acc: Tensor, w: float, mode: int) -> None:
    """Trapezoid history sums (lbm_history_accumulate; model.py:257-277):
    mode 0 records cur as prev, mode 1 adds w (cur + prev) to the FP64 acc."""
    keep = _Keep()
    check(lib().lbm_history_accumulate(_prec(cur), acc.numel(), _p(keep(cur)), _p(_w(prev)),
                                       _p(_w(acc)), float(w), int(mode), _st()),
          "lbm_history_accumulate")


@history_accumulate.register_fake
def _(cur, prev, acc, w, mode):
    return None


@torch.library.custom_op(f"{NS_}::link_copy_", mutates_args=("dst",))
def link_copy_(dst: Tensor, src: Tensor) -> None:
    """dst <- src (same shape and dtype, contiguous) by SM loads and stores
    over the CPU-GPU link (lbm_link_copy); each tensor on the GPU or in
    pinned host memory."""
    if dst.shape != src.shape or dst.dtype != src.dtype:
        raise ValueError("link_copy_: shapes and dtypes must match")
    _w(dst)
    if not src.is_contiguous():
        raise ValueError("link_copy_: src must be contiguous")
    if dst.device.type == "cpu" and not dst.is_pinned():
        raise ValueError("link_copy_: host tensors must be pinned")
    if src.device.type == "cpu" and not src.is_pinned():
        raise ValueError("link_copy_: host tensors must be pinned")
    check(lib().lbm_link_copy(_p(dst), _p(src), dst.numel() * dst.element_size(), _st()),
          "lbm_link_copy")


@link_copy_.register_fake
def _(dst, src):
    return None


OPS = ("gauss_legendre", "legendre_tables", "fft_twiddles", "gravity_wave_matrices",
       "batched_inverse", "fourier_forward", "fourier_inverse", "legendre_analysis",
       "legendre_synthesis", "tendency_grid", "implicit_step", "tendency_grid_adjoint",
       "implicit_step_adjoint", "stepper_run", "stepper_prime", "stepper_colsum",
       "stepper_flush", "history_accumulate", "link_copy_")
