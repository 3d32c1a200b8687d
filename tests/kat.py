"""Analytic known-answer cases shared by the oracle and GPU KAT tests.

plane_wave: the free field (theory 1 with Lambda_Mode = 0, h = 0: V' = M^2 phi)
    from phi = A cos(k.x), pi = 0.  The lattice Laplacian's eigenvalue on the
    wave is -sum_d (4/a^2) sin^2(pi n_d / N), so the mode is a harmonic
    oscillator with w^2 = M^2 + sum_d (4/a^2) sin^2(pi n_d / N); the
    reference's leapfrog (half kick first) maps it exactly to
    phi_n = A cos(k.x) cos(n th), cos th = 1 - (w h)^2 / 2, and after n steps
    pi holds pi_{n-1/2} = (phi_n - phi_{n-1}) / h.
homogeneous_ode: a uniform field sees no Laplacian: phi'' = -V'(phi), solved
    to 1e-13 by an explicit Runge-Kutta (DOP853); the leapfrog error at fixed
    T falls as h^2.
"""
import numpy as np

A_WAVE = 0.7
MODE = (1, 2, 0)
KAPPA = 3.0 ** 0.5


def wave_params(N: int = 16, a: float = 0.25, dt: float = 0.08) -> dict:
    return dict(N=N, a=a, dt=dt, theory=1, mass_mode=1, m_sqr=1.0, lambda_mode=0, h=0.0)


def plane_wave(N: int, a: float):
    """[z][y][x] initial phi of the wave."""
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    return A_WAVE * np.cos(2 * np.pi * (MODE[0] * x + MODE[1] * y + MODE[2] * z) / N)


def plane_wave_exact(N: int, a: float, h: float, steps: int):
    """phi_n and pi_{n-1/2} of the leapfrog after `steps` steps."""
    w2 = 1.0 + sum(4.0 / a ** 2 * np.sin(np.pi * nd / N) ** 2 for nd in MODE)
    th = np.arccos(1.0 - w2 * h * h / 2.0)
    f0 = plane_wave(N, a)
    return f0 * np.cos(steps * th), f0 * (np.cos(steps * th) - np.cos((steps - 1) * th)) / h


def phi6_force(f):
    """V'(Phi) of the phi^6 potential in the reference's parameterisation
    (theory 0: Mass_Mode 1, M^2 = 1, Lambda_Mode -1, Kappa = sqrt(3), Nc = 1)."""
    return (1.0 - f * f / 6.0 + (f * f / KAPPA) ** 2 / 120.0) * f


def ode_reference(f0: float, T: float) -> float:
    from scipy.integrate import solve_ivp
    sol = solve_ivp(lambda t, u: [u[1], -phi6_force(u[0])], (0.0, T), [f0, 0.0], method="DOP853", rtol=1e-13,
                    atol=1e-13)
    return float(sol.y[0, -1])


def phi6_params(N: int, a: float, h: float) -> dict:
    return dict(N=N, a=a, dt=h / a, theory=0, mass_mode=1, m_sqr=1.0, lambda_mode=-1, kappa=KAPPA)
