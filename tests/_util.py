"""Shared helpers for the test suite (seeded inputs, error metrics)."""
import numpy as np


def crand(rng, shape, dist="uniform"):
    if dist == "uniform":  # genComplex: re, im ~ U[-1, 1] (Fourier.hs:50-51)
        return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def fp32_bound(n, c=4.0):
    """c * eps32 * log2 N relative-L2 bound for an FP32 transform of length n."""
    return c * 2.0 ** -24 * max(1.0, np.log2(max(n, 2)))
