"""lbm_isca_gb300 -- GB300-native dynamical-core hot path for PyLBM-Isca.

Drop-in for the ``pylbm_isca`` package facade (pylbm_isca/__init__.py:21-32):
``Spectral``, ``VerticalGrid``, ``LBM``, ``Config``, ``State`` and the backend
helpers keep the reference's names, signatures and array conventions, but
every object lives on a CUDA device and every transform, tendency and
implicit step runs in the hand-written sm_103a kernels of the lbm_gb300
library (``lbm_isca_gb300/csrc``, C ABI in ``include/lbm_gb300.h``).

Importing the package needs neither a GPU nor the compiled library; the
first object that needs the kernels loads the library and raises if it is
missing or no CUDA device is visible (there is no CPU fallback).
"""

from .constants import IMAX, JMAX, KMAX, NMAX

__version__ = "0.1.0"

_LAZY = {
    "Spectral": ("spectral", "Spectral"),
    "VerticalGrid": ("vertical", "VerticalGrid"),
    "LBM": ("model", "LBM"),
    "Config": ("model", "Config"),
    "State": ("state", "State"),
    "BatchedSpectral": ("ensemble", "BatchedSpectral"),
    "EnsembleForcing": ("ensemble", "EnsembleForcing"),
    "make_ensemble_model": ("ensemble", "make_ensemble_model"),
    "gpu_available": ("backend", "gpu_available"),
    "device_name": ("backend", "device_name"),
    "asnumpy": ("backend", "asnumpy"),
    "resolve": ("backend", "resolve"),
    "MJOForcing": ("forcing", "MJOForcing"),
}

__all__ = ["Spectral", "VerticalGrid", "LBM", "Config", "State", "IMAX", "JMAX", "KMAX",
           "NMAX", "gpu_available", "device_name", "asnumpy", "resolve",
           "BatchedSpectral", "EnsembleForcing", "make_ensemble_model", "MJOForcing"]


def __getattr__(name):
    if name in _LAZY:
        import importlib
        mod, attr = _LAZY[name]
        return getattr(importlib.import_module(f".{mod}", __name__), attr)
    raise AttributeError(name)
