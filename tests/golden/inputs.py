"""Seeded lattice inputs that are bit-identical on every platform.

Parity fixtures compare FP64 fields bit for bit, so their inputs must not
depend on libm or on a numpy version: values come from SplitMix64 (integer
arithmetic), mapped to uniforms k/2^53 and summed (exact IEEE additions in a
fixed order), then smoothed by nearest-neighbour averaging (again fixed-order
IEEE additions and multiplications).  The result is a zero-mean,
roughly Gaussian fluctuation of unit-order amplitude with suppressed high-k
content, added to a homogeneous value.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(idx: np.ndarray, seed: int) -> np.ndarray:
    """SplitMix64 of (seed, index): one independent 64-bit word per index."""
    with np.errstate(over="ignore"):
        z = idx.astype(np.uint64) + np.uint64((seed * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)
        z = z * np.uint64(0x9E3779B97F4A7C15) + np.uint64(0x632BE59BD9B4E5B5)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniforms(n: int, seed: int, stream: int) -> np.ndarray:
    """n uniforms in [0,1), exactly representable (multiples of 2^-53)."""
    idx = np.arange(n, dtype=np.uint64) * np.uint64(4) + np.uint64(stream)
    return (splitmix64(idx, seed) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def noise(shape, seed: int, stream: int = 0) -> np.ndarray:
    """Zero-mean unit-variance Irwin-Hall(4) noise, then two smoothing passes."""
    n = int(np.prod(shape))
    g = np.zeros(n)
    for k in range(4):
        g = g + uniforms(n, seed, 4 * stream + k)
    g = (g - 2.0) * 1.7320508075688772  # variance of the sum of 4 U(0,1) is 1/3
    g = g.reshape(shape)
    axes = tuple(range(g.ndim - 3, g.ndim))
    for _ in range(2):
        s = g * 2.0
        for ax in axes:
            s = s + np.roll(g, 1, axis=ax)
            s = s + np.roll(g, -1, axis=ax)
        g = s * 0.125
    return g


def lattice_fields(N: int, Nc: int = 1, seed: int = 0, phi0: float = 2.449489742783178,
                   amp_phi: float = 1.2, amp_pi: float = 1.2):
    """phi, pi as [Nc][z][y][x] float64: homogeneous phi0 (component 0) plus
    smoothed noise (standard deviation about 0.25 * amp); pi is pure noise."""
    phi = noise((Nc, N, N, N), seed, 0) * amp_phi
    phi[0] = phi[0] + phi0
    pi = noise((Nc, N, N, N), seed, 1) * amp_pi
    return phi, pi
