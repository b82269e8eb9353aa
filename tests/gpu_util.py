"""Helpers shared by the GPU tests."""
import numpy as np
import pytest


def need_gpu():
    try:
        import torch
    except Exception:  # pragma: no cover
        pytest.skip("torch unavailable")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def fp():
    """The product package with its native library built."""
    import fastpcc_gb300 as F
    F.build()
    return F


def relerr(y, y64):
    y = np.atleast_2d(np.asarray(y, np.float64))
    y64 = np.atleast_2d(np.asarray(y64, np.float64))
    return float(np.max(np.max(np.abs(y - y64), axis=1) / np.max(np.abs(y64), axis=1)))
