"""Deterministic inputs of the golden sweeps, shared by make_golden.py (which
runs the reference on them) and the tests (which run this package on them):
formulas instead of stored arrays, so that the fixtures hold only the
parameters and digests of the reference's outputs.

TEST INFRASTRUCTURE."""
import hashlib

import numpy as np

NDV = -9999.0


def drift_rasters(nr, nc, k, phase):
    """k rasters [nr, nc]: smooth values in [-1000, 1000] with no-data cells
    on a lattice pattern, and cells just inside (-9999.05) and just outside
    (-9998.8) np.isclose's reach of the no-data value."""
    i, j = np.meshgrid(np.arange(nr), np.arange(nc), indexing="ij")
    out = []
    for r in range(k):
        a = 1000.0 * np.sin(0.37 * (r + 1) * i + 0.11 * j + phase + r)
        a[(i * 7 + j * 3 + r) % 13 == 0] = NDV
        a[(i * 5 + j * 11 + r) % 29 == 0] = NDV - 0.05
        a[(i * 3 + j * 5 + r) % 31 == 0] = NDV + 1.2
        out.append(a)
    return out


def cell_mask(n):
    """A fixed selection of about 60% of n cells."""
    return (np.arange(n) * 7919) % 10 < 6


def digest(a):
    """SHA-256 of an array's float64 little-endian bytes."""
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).digest()
