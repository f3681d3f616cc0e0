"""Shared comparison helpers for the parity tests."""
import numpy as np


def rel_err(gpu, ref):
    """Max |gpu - ref| over the array divided by max |ref| (the per-component error metric)."""
    gpu = np.asarray(gpu)
    ref = np.asarray(ref)
    assert gpu.shape == ref.shape, (gpu.shape, ref.shape)
    assert np.isfinite(ref).all(), "reference has non-finite values"
    scale = np.abs(ref).max()
    d = np.abs(gpu - ref).max()
    if scale == 0.0:
        return float(d)
    return float(d / scale)


def per_comp_rel_err(gpu, ref):
    return [rel_err(gpu[c], ref[c]) for c in range(ref.shape[0])]
