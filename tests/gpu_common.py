"""Shared helpers for the GPU parity tests: seeded inputs and error metrics."""
import math

import numpy as np

from oracle import oracle as O


def peak_norm_err(gpu, ref):
    ref = np.asarray(ref)
    scale = float(np.max(np.abs(ref)))
    return float(np.max(np.abs(np.asarray(gpu) - ref))) / (scale if scale > 0 else 1.0)


def random_batch(rng, n, gnx, du, margin=8, w_max=0.0, weights=True):
    """Samples uniform over the usable grid, random weights and visibilities."""
    half = (gnx / 2 - margin) * du
    u = rng.uniform(-half, half, n)
    v = rng.uniform(-half, half, n)
    w = rng.uniform(-w_max, w_max, n) if w_max > 0 else np.zeros(n)
    wt = (rng.uniform(0.5, 2.0, n) if weights else np.ones(n)).astype(np.float32)
    vis = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    return u, v, w, wt, vis


def small_geometry(nx=64, cell=1e-4):
    return O.Geometry(nx, nx, cell, cell)


def arcsec(a):
    return math.radians(a / 3600.0)
