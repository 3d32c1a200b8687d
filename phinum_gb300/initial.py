"""Seeded Gaussian initial fields with the reference's mode recipe.

Follows SetInitialConditions for `initialize 3`, static box
(initialconditions.cpp:83-698): for every lattice momentum p (components
(2/a) sin(pi n/N)), occupation n = Noise below the cutoff scale2 on |p| and 0
above; Omega = sqrt(p^2 + M2_long) with M2_long = M_sqr (renormalization.cpp:17);
field mode A = |g1| sqrt(n) e^{i th1} / sqrt(Omega), momentum mode
E = |g2| sqrt(n) e^{i th2} sqrt(Omega); the inverse transform (unnormalised,
divided by L^3, clusterfft.cpp:148-182) times sqrt(L^3) plus the homogeneous
values phi0, pi0 (initialconditions.cpp:638-681).

Random numbers come from numpy's PCG64 instead of drand48, and Hermitian
symmetry is imposed by the inverse real FFT, so the fields are statistically,
not bitwise, equivalent to the reference's.
"""
from __future__ import annotations

import numpy as np


def lattice_momenta(N: int, a: float) -> np.ndarray:
    n = np.arange(N)
    return 2.0 / a * np.sin(np.pi * n / N)


def gaussian_fields(N: int, a: float = 0.25, phi0: float = 6.0 ** 0.5, pi0: float = 0.0, m_sqr: float = 1.0,
                    noise: float = 3.0, scale2: float = 2 * np.pi, seed: int = 0):
    """phi, pi as [z][y][x] float64 arrays."""
    rng = np.random.default_rng(seed)
    p = lattice_momenta(N, a)
    px = p[: N // 2 + 1][None, None, :]
    py = p[None, :, None]
    pz = p[:, None, None]
    psqr = px * px + py * py + pz * pz
    occ = np.where(np.sqrt(psqr) < scale2, noise, 0.0)
    omega = np.sqrt(psqr + m_sqr)
    shape = psqr.shape
    L3 = (N * a) ** 3

    def modes(scale):
        g = np.abs(rng.standard_normal(shape))
        th = rng.uniform(0.0, 2 * np.pi, shape)
        return (g * np.sqrt(occ) * scale) * np.exp(1j * th)

    A = modes(1.0 / np.sqrt(omega))
    E = modes(np.sqrt(omega))
    norm = N ** 3 / np.sqrt(L3)  # irfftn divides by N^3; the reference divides by L^3 and multiplies by sqrt(L^3)
    phi = np.fft.irfftn(A, s=(N, N, N), axes=(0, 1, 2)) * norm + phi0
    pi = np.fft.irfftn(E, s=(N, N, N), axes=(0, 1, 2)) * norm + pi0
    return phi, pi
