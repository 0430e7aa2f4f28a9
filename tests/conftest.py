"""Shared pytest configuration: the `gpu` marker and repo-root imports."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA device and the compiled lbm_gb300 library")
    config.addinivalue_line("markers", "slow: long CPU-only run (oracle trajectories)")


def golden(name):
    """Load one golden .npz fixture produced by tests/golden/make_golden.py."""
    return np.load(os.path.join(GOLDEN, name))


def unpack(x, M):
    """[..., NS, (K)] packed n>=m -> [..., M, M, (K)] rectangle (zeros n<m)."""
    x = np.asarray(x)
    mm, nn = np.nonzero(np.triu(np.ones((M, M), dtype=bool)))
    NS = mm.size
    if x.shape[-1] == NS:
        out = np.zeros(x.shape[:-1] + (M, M), dtype=x.dtype)
        out[..., mm, nn] = x
    else:
        out = np.zeros(x.shape[:-2] + (M, M, x.shape[-1]), dtype=x.dtype)
        out[..., mm, nn, :] = x
    return out


def pack(x, M):
    x = np.asarray(x)
    mm, nn = np.nonzero(np.triu(np.ones((M, M), dtype=bool)))
    if x.shape[-2:] == (M, M):
        return x[..., mm, nn]
    return x[..., mm, nn, :]


def relerr(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))
