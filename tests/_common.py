"""Shared helpers of the test-suite: seeded inputs and the parity metric."""

import numpy as np

# Relative parity tolerance of the FP64 paths: max|gpu - oracle| / max|oracle|.
RTOL = 1e-12


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b))
    if den == 0.0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b)) / den)


def seeded_material(nelem, seed):
    """Per-element K ~ U[0.5, 1.5], G ~ U[0.25, 0.75]."""
    rng = np.random.default_rng(seed)
    K = rng.uniform(0.5, 1.5, nelem)
    G = rng.uniform(0.25, 0.75, nelem)
    return K, G


def seeded_field(shape, seed, amp=1e-3):
    rng = np.random.default_rng(seed)
    return rng.uniform(-amp, amp, shape)


def to_np(t):
    return t.detach().cpu().numpy() if hasattr(t, "detach") else np.asarray(t)
