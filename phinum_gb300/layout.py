"""Host-side conversions to and from the reference's field layout.

Reference layout (lattice.cpp:76-78, util.cpp:34-37): Nc*N*N*(N+2) values,
index Nc*(x + N*y + N*N*z) + a, z-slabs 0 and N+1 are ghost copies of slabs N
and 1 (what Communication::exchange() leaves with one rank).
"""
from __future__ import annotations

import numpy as np


def to_ref_layout(field: np.ndarray, Nc: int | None = None) -> np.ndarray:
    """[Nc][z][y][x] (or [z][y][x]) -> flat reference layout, ghosts filled."""
    f = np.asarray(field, dtype=np.float64)
    if f.ndim == 3:
        f = f[None]
    nc, n = f.shape[0], f.shape[1]
    out = np.empty((n + 2, n, n, nc))
    out[1:n + 1] = np.moveaxis(f, 0, -1)
    out[0] = out[n]
    out[n + 1] = out[1]
    return out.reshape(-1)


def from_ref_layout(flat: np.ndarray, N: int, Nc: int = 1) -> np.ndarray:
    """Flat reference layout -> [Nc][z][y][x] interior."""
    f = np.asarray(flat).reshape(N + 2, N, N, Nc)[1:N + 1]
    return np.ascontiguousarray(np.moveaxis(f, -1, 0))
