"""Shared helpers of the test-suite: seeded smooth random fields and error
measures (relative L2 and bitwise equality)."""
from __future__ import annotations

import numpy as np


def smooth_field(shape, seed, amp=1.0, modes=4):
    """Sum of low-frequency sinusoids plus 5 % white noise, seeded."""
    rng = np.random.default_rng(seed)
    grids = np.meshgrid(*[np.linspace(0, 1, n, endpoint=False) for n in shape], indexing="ij")
    f = np.zeros(shape, dtype=np.float64)
    for _ in range(modes):
        k = rng.integers(1, 4, size=len(shape))
        ph = rng.uniform(0, 2 * np.pi, size=len(shape))
        term = np.ones(shape)
        for d in range(len(shape)):
            term = term * np.sin(2 * np.pi * k[d] * grids[d] + ph[d])
        f += rng.uniform(-1, 1) * term
    f += 0.05 * rng.standard_normal(shape)
    return (amp * f / max(1e-12, np.abs(f).max())).astype(np.float32)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return num / den if den > 0 else num


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.dtype == np.float32:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    return np.array_equal(a, b)
