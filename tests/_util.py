"""Shared helpers for the test suite."""
import numpy as np


def rel_err(a, b):
    """max |a - b| / max |b| (norm-wise relative error)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.abs(b).max()
    if den == 0:
        return float(np.abs(a).max())
    return float(np.abs(a - b).max() / den)
