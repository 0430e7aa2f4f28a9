"""Device selection for the GB300 path (mirrors pylbm_isca/backend.py:48-114).

The reference maps a device string to an array module (numpy / cupy).  Here
every object lives on one CUDA device as torch tensors driven by the
lbm_gb300 kernels, so ``resolve`` returns a ``torch.device``.  Accepted
values: ``"gb300"``, ``"gpu"``, ``"cuda"``, ``"cuda:N"``, ``"auto"`` /
``None`` (honouring ``$LBM_DEVICE``).  A GPU request without a CUDA device
raises ``RuntimeError`` (backend.py:69-74); ``"cpu"``/``"numpy"`` raise
``RuntimeError`` too, because this package has no CPU path (use the
reference package for CPU runs); anything else raises ``ValueError``
(backend.py:77).
"""

from __future__ import annotations

import os

import numpy as np
import torch

_GPU_NAMES = ("gb300", "gpu", "cuda")


def gpu_available():
    return torch.cuda.is_available()


def resolve(device=None):
    if isinstance(device, torch.device):
        if device.type != "cuda":
            raise RuntimeError("the GB300 path runs on CUDA devices only")
        if not gpu_available():
            raise RuntimeError("CUDA device requested but none is available")
        return device
    if device is None or str(device).lower() == "auto":
        env = os.environ.get("LBM_DEVICE", "").strip().lower()
        if env and env != "auto":
            return resolve(env)
        return resolve("gb300")
    d = str(device).lower()
    if d in _GPU_NAMES or d.startswith("cuda:"):
        if not gpu_available():
            raise RuntimeError(
                f"device={device!r} requested but no CUDA device is visible; the GB300 "
                "path has no CPU fallback")
        if d.startswith("cuda:"):
            return torch.device(d)
        return torch.device("cuda", torch.cuda.current_device())
    if d in ("cpu", "numpy"):
        raise RuntimeError(
            "the GB300 package has no CPU path; use the reference pylbm_isca for "
            "device='cpu'")
    raise ValueError(f"unknown device {device!r}")


def to_device(x, device, dtype=torch.float64):
    """Host (numpy) or device array -> contiguous tensor on `device`."""
    if isinstance(x, torch.Tensor):
        t = x.to(device=device)
        if dtype is not None and not torch.is_complex(t) and t.dtype != dtype:
            t = t.to(dtype)
        return t.contiguous()
    a = np.asarray(x)
    if np.iscomplexobj(a):
        return torch.as_tensor(np.ascontiguousarray(a, dtype=np.complex128), device=device)
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=device).to(
        dtype if dtype is not None else torch.float64)


def asnumpy(x):
    """Bring an array to the host as numpy (no-op for numpy input)."""
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def get_array_module(*arrays):
    return torch


def device_name(dev=None):
    return "gb300"


def synchronize(dev=None):
    if gpu_available():
        torch.cuda.synchronize()


def stream_handle(stream=None):
    """Raw cudaStream_t of a torch stream (default: the current stream)."""
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
