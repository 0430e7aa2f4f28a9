"""The C-ABI library builds, loads and exports every entry point that
include/lbm_gb300.h declares (no compute calls: runs without a GPU)."""

import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "lbm_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set(re.findall(r"\b(lbm_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_the_entry_points():
    names = declared_symbols()
    for must in ("lbm_legendre_tables", "lbm_fourier_forward", "lbm_tendency_grid",
                 "lbm_implicit_step", "lbm_stepper_run", "lbm_graph_capture"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from lbm_isca_gb300.build import build
    path = build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    lib.lbm_version.restype = ctypes.c_char_p
    assert lib.lbm_version().startswith(b"lbm_gb300")


def test_bad_arguments_are_rejected_without_a_device():
    """Argument validation happens before any CUDA call."""
    from lbm_isca_gb300 import _lib
    L = _lib.lib()
    assert L.lbm_gauss_legendre(1, None, None, None) == _lib.LBM_ERR_ARG
    assert L.lbm_fourier_forward(_lib.LBM_F64, 1, 32, 100, 1, 21, None, None, None, None,
                                 None) == _lib.LBM_ERR_ARG
    assert L.lbm_stepper_run(None, None, 1, None) == _lib.LBM_ERR_ARG
    assert L.lbm_batched_inverse(1, 65, None, None, None, None) == _lib.LBM_ERR_ARG


def test_noalloc_stepper_rejects_oversized_cases_without_a_device():
    """The static-scratch stepper checks its size before any CUDA call."""
    import ctypes as C
    from lbm_isca_gb300 import _lib
    L = _lib.lib()
    d = _lib.StepperDesc()
    d.prec, d.nmem, d.nlat, d.nlon, d.nmax, d.kmax, d.nsets = _lib.LBM_F32, 6, 64, 128, 42, 20, 1
    ctl = (_lib.StepCtl * 1)()
    assert L.lbm_stepper_run_noalloc(C.byref(d), ctl, 1, None) == _lib.LBM_ERR_SCRATCH
    d.nmem = 0
    assert L.lbm_stepper_run_noalloc(C.byref(d), ctl, 1, None) == _lib.LBM_ERR_ARG
    assert L.lbm_stepper_run_noalloc(None, ctl, 1, None) == _lib.LBM_ERR_ARG
    # a negative or unsupported longitude count would make the area's size
    # negative: rejected before the size comparison
    d.nmem = 1
    for nlon in (-128, 0, 96):
        d.nlon = nlon
        assert L.lbm_stepper_run_noalloc(C.byref(d), ctl, 1, None) == _lib.LBM_ERR_ARG


def test_io_and_setup_entry_points_reject_bad_arguments_without_a_device():
    """History packing and basic-state column kernels validate before any
    CUDA call."""
    import ctypes as C
    from lbm_isca_gb300 import _lib
    L = _lib.lib()
    VP = C.c_void_p
    fake = VP(16)                      # never dereferenced: rejected first
    ptrs = (VP * 8)(*([fake] * 8))
    nulls = (VP * 8)()
    assert L.lbm_grads_records(0, 20, ptrs, 1, 100.0, 12.0, fake, None) == _lib.LBM_ERR_ARG
    assert L.lbm_grads_records(8192, 20, nulls, 1, 100.0, 12.0, fake, None) == _lib.LBM_ERR_ARG
    assert L.lbm_grads_records(8192, 20, ptrs, 1, 100.0, 0.0, fake, None) == _lib.LBM_ERR_ARG
    assert L.lbm_z2ps(0, 17, fake, None, fake, fake, None) == _lib.LBM_ERR_ARG
    assert L.lbm_z2ps(10, 1, fake, None, fake, fake, None) == _lib.LBM_ERR_ARG
    assert L.lbm_spline(10, 65, 5, fake, fake, fake, fake, 0, 0, -999.0, None) == _lib.LBM_ERR_ARG
    assert L.lbm_spline(10, 17, 0, fake, fake, fake, fake, 0, 0, -999.0, None) == _lib.LBM_ERR_ARG
    assert L.lbm_zonal_filter(32, 64, 20, fake, 3, None) == _lib.LBM_ERR_ARG
    assert L.lbm_zonal_filter(32, 64, 20, None, 1, None) == _lib.LBM_ERR_ARG
