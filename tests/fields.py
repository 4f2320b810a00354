"""Seeded synthetic fields with the shapes and spectra of the benchmark configurations.

All arrays are Fortran-ordered (x fastest), like the reference's fields.
"""
import numpy as np


def random_modes(n, nmodes, kmax, seed, z_nonperiodic=False, profile=False):
    """Sum of nmodes Fourier modes with integer wavevectors |k_i| <= kmax, amplitudes
    N(0,1)*|k|^(-5/6) and random phases on [0, 2pi)^3 (z on [0, 1] when z_nonperiodic,
    times tanh(4(z - 0.5)) when profile)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    x = np.arange(nx) * 2 * np.pi / nx
    y = np.arange(ny) * 2 * np.pi / ny
    if z_nonperiodic:
        zz = np.linspace(0.0, 1.0, nz)
        z = 2 * np.pi * zz
    else:
        z = np.arange(nz) * 2 * np.pi / nz
    f = np.zeros((nx, ny, nz), order="F")
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    for _ in range(nmodes):
        k = np.zeros(3)
        while not np.any(k):
            k = rng.integers(-kmax, kmax + 1, size=3)
        amp = rng.standard_normal() * np.linalg.norm(k) ** (-5.0 / 6.0)
        ph = rng.uniform(0, 2 * np.pi)
        f += amp * np.cos(k[0] * X + k[1] * Y + k[2] * Z + ph)
    if profile:
        f *= np.tanh(4 * (np.linspace(0.0, 1.0, nz) - 0.5))[None, None, :]
    return np.asfortranarray(f)


def relerr(a, b):
    """Normwise relative difference max|a-b| / max|b|."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))
