"""ctypes binding of the lbm_gb300 C ABI (include/lbm_gb300.h).

The library is loaded on first use.  There is no fallback: if the compiled
library is missing or no CUDA device is present, every call raises.
"""

from __future__ import annotations

import ctypes as C
import os

from .build import LIBPATH

LBM_OK, LBM_ERR_ARG, LBM_ERR_LAUNCH, LBM_ERR_SINGULAR, LBM_ERR_NONFINITE = 0, 1, 2, 3, 4
LBM_ERR_SCRATCH = 5
LBM_NOALLOC_SCRATCH_BYTES = 32 << 20
LBM_F64, LBM_F32 = 0, 1
_STATUS = {LBM_ERR_ARG: "bad argument or unsupported size",
           LBM_ERR_LAUNCH: "CUDA launch/runtime failure",
           LBM_ERR_SINGULAR: "singular matrix", LBM_ERR_NONFINITE: "non-finite value"}

VP = C.c_void_p
I32 = C.c_int
F64 = C.c_double


class TendGridArgs(C.Structure):
    _fields_ = ([("nmem", I32), ("nlat", I32), ("nlon", I32), ("kmax", I32),
                 ("strictly_linear", I32), ("kappa", F64), ("epsvt", F64), ("rair", F64)]
                + [(n, VP) for n in ("dsig", "sigm", "alpha", "w3", "wP", "cpg", "sig", "ww",
                                     "tmtx", "tref", "ub", "vb", "tb", "qb", "tvb", "absvor",
                                     "divb", "x5b", "sdotb", "pixb", "piyb", "psb", "u", "v",
                                     "t", "q", "vor", "div", "pix", "piy", "ps", "frc_t",
                                     "frc_ps", "frc_q")]
                + [("frc_t_stride", C.c_int64), ("frc_ps_stride", C.c_int64),
                   ("frc_q_stride", C.c_int64)]
                + [(n, VP) for n in ("fu", "fv", "ke", "gt", "xu", "xv", "g", "yu", "yv",
                                     "gt_pi", "omega", "sdot", "lin_u", "lin_v")])


class TendAdjArgs(C.Structure):
    _fields_ = ([("nmem", I32), ("nlat", I32), ("nlon", I32), ("kmax", I32),
                 ("kappa", F64), ("epsvt", F64), ("rair", F64)]
                + [(n, VP) for n in ("dsig", "sigm", "alpha", "w3", "wP", "cpg", "ww", "tmtx",
                                     "tref", "ub", "vb", "tb", "qb", "tvb", "absvor", "divb",
                                     "x5b", "sdotb", "pixb", "piyb", "u0", "v0", "a_fu", "a_fv",
                                     "a_ke", "a_gt", "a_xu", "a_xv", "a_g", "a_yu", "a_yv",
                                     "a_gt_pi", "a_u", "a_v", "a_t", "a_q", "a_vor", "a_div",
                                     "a_pix", "a_piy")])


class ImplicitArgs(C.Structure):
    _fields_ = ([("nmem", I32), ("nmax", I32), ("kmax", I32), ("dt", F64)]
                + [(n, VP) for n in ("lap", "kv", "kd", "ktt", "kq", "ww", "tmtx", "gg",
                                     "dsig", "minv", "vd_vor", "vd_div", "vd_t", "vd_q",
                                     "p_vor", "p_div", "p_t", "p_pi", "p_q", "w_vor", "w_div",
                                     "w_t", "w_pi", "w_q", "n_vor", "n_div", "n_t", "n_pi",
                                     "n_q")])


class ImplicitAdjArgs(C.Structure):
    _fields_ = ([("nmem", I32), ("nmax", I32), ("kmax", I32), ("dt", F64)]
                + [(n, VP) for n in ("lap", "kv", "kd", "ktt", "kq", "ww", "tmtx", "gg",
                                     "dsig", "minv", "vd_vor", "vd_div", "vd_t", "vd_q",
                                     "an_vor", "an_div", "an_t", "an_pi", "an_q", "ap_vor",
                                     "ap_div", "ap_t", "ap_pi", "ap_q", "aw_vor", "aw_div",
                                     "aw_t", "aw_pi", "aw_q")])


class StepperDesc(C.Structure):
    _fields_ = ([(n, I32) for n in ("prec", "nmem", "nlat", "nlon", "nmax", "kmax", "nsets",
                                    "strictly_linear")]
                + [("vd_on", I32 * 4), ("frc_shared", I32),
                   ("kappa", F64), ("epsvt", F64), ("robert", F64)]
                + [(n, VP) for n in ("symp", "symh", "tw", "jfac", "vert", "b3", "bsd", "b2",
                                     "lap", "invlap", "nn1a", "kv", "kd", "ktt", "kq", "ww",
                                     "tmtx", "minv", "vdiff", "frc3", "frcs", "dft", "sa3", "sas",
                                     "sb3", "psa", "psb", "sf", "sfs", "af", "afs", "tend",
                                     "tends", "grid6", "grid9")]
                + [("err", C.POINTER(I32)), ("err_member", C.POINTER(I32)),
                   ("legendre", I32), ("tc_anal", VP), ("tc_synth", VP), ("tc_off", I32),
                   ("tc_g", I32), ("tc_dft", VP)])


class StepCtl(C.Structure):
    _fields_ = [("dt", F64), ("set", I32), ("ps_mode", I32), ("ra_mode", I32), ("pad", I32)]


_SIGS = {
    "lbm_version": (C.c_char_p, []),
    "lbm_gauss_legendre": (I32, [I32, VP, VP, VP]),
    "lbm_legendre_tables": (I32, [I32, I32, VP, VP, VP, VP]),
    "lbm_fft_twiddles": (I32, [I32, VP, VP]),
    "lbm_gravity_wave_matrices": (I32, [I32, I32, F64, VP, VP, VP, VP, VP, VP, VP]),
    "lbm_batched_inverse": (I32, [I32, I32, VP, VP, VP, VP]),
    "lbm_fourier_forward": (I32, [I32, I32, I32, I32, I32, I32, VP, VP, VP, VP, VP]),
    "lbm_fourier_inverse": (I32, [I32, I32, I32, I32, I32, I32, VP, VP, VP, VP, VP]),
    "lbm_legendre_analysis": (I32, [I32, I32, I32, I32, I32, VP, VP, I32, VP, VP, I32, F64,
                                    VP, I32, VP, VP]),
    "lbm_legendre_synthesis": (I32, [I32, I32, I32, I32, I32, VP, VP, I32, VP, VP, VP, I32,
                                     VP, F64, VP, VP]),
    "lbm_tendency_grid": (I32, [I32, C.POINTER(TendGridArgs), VP]),
    "lbm_implicit_step": (I32, [I32, C.POINTER(ImplicitArgs), VP]),
    "lbm_tendency_grid_adjoint": (I32, [I32, C.POINTER(TendAdjArgs), VP]),
    "lbm_implicit_step_adjoint": (I32, [I32, C.POINTER(ImplicitAdjArgs), VP]),
    "lbm_stepper_prime": (I32, [C.POINTER(StepperDesc), VP]),
    "lbm_stepper_run": (I32, [C.POINTER(StepperDesc), C.POINTER(StepCtl), I32, VP]),
    "lbm_stepper_launch": (I32, [C.POINTER(StepperDesc), C.POINTER(StepCtl), I32, VP]),
    "lbm_stepper_flush": (I32, [C.POINTER(StepperDesc), I32, VP]),
    "lbm_stepper_colsum": (I32, [C.POINTER(StepperDesc), VP]),
    "lbm_graph_capture": (I32, [C.POINTER(StepperDesc), C.POINTER(StepCtl), I32, VP,
                                C.POINTER(VP)]),
    "lbm_graph_launch": (I32, [VP, VP]),
    "lbm_graph_destroy": (I32, [VP]),
    "lbm_stepper_run_noalloc": (I32, [C.POINTER(StepperDesc), C.POINTER(StepCtl), I32, VP]),
    "lbm_history_accumulate": (I32, [I32, C.c_int64, VP, VP, VP, F64, I32, VP]),
    "lbm_link_copy": (I32, [VP, VP, C.c_int64, VP]),
    "lbm_grads_records": (I32, [C.c_int64, I32, C.POINTER(VP), I32, F64, F64, VP, VP]),
    "lbm_z2ps": (I32, [C.c_int64, I32, VP, VP, VP, VP, VP]),
    "lbm_spline": (I32, [C.c_int64, I32, I32, VP, VP, VP, VP, I32, I32, F64, VP]),
    "lbm_zonal_filter": (I32, [I32, I32, I32, VP, I32, VP]),
}

_LIB = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(
                f"lbm_gb300 native library not found at {LIBPATH}; build it with "
                "`python -m lbm_isca_gb300.build` (there is no CPU fallback)")
        h = C.CDLL(LIBPATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = h
    return _LIB


def check(status, what):
    if status != LBM_OK:
        raise RuntimeError(f"{what} failed: {_STATUS.get(status, status)} (status {status})")


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    return None if t is None else VP(t.data_ptr())
