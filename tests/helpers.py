"""Shared comparison helpers for the parity tests."""
import numpy as np


def normwise(a, b):
    """max |a - b| / max |b| (the FFT-inclusive tolerance is normwise)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def relerr(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def pixelwise(a, b):
    """max over pixels of |a - b| / |b| (pre-FFT tolerance)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))
