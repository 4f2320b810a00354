"""Seeded synthetic fields with the shapes and spectra of the benchmark configurations.

The reference's input data (HIT restart files, DNS fields) are not available; these
generators stand in for them.  Arrays are Fortran-ordered (x fastest), like the
reference's fields.
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


def hit_initial_field(n, seed=4, kp=4.0, urms=1.0):
    """Seeded solenoidal-spectrum field on [0, 2pi)^3: E(k) ~ k^4 exp(-2 (k/kp)^2), random
    phases, scaled to u_rms; w returned on nz+1 edge planes (plane nz+1 = plane 1).  The
    projection inside init_fields makes it discretely divergence free."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n, 1.0 / n)
    KX, KY, KZ = np.meshgrid(k, k, k, indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    kk[0, 0, 0] = 1.0
    E = kk ** 4 * np.exp(-2.0 * (kk / kp) ** 2)
    amp = np.sqrt(E / (4 * np.pi * kk ** 2))
    amp[0, 0, 0] = 0.0
    amp[np.abs(KX) >= n // 3] = 0.0
    amp[np.abs(KY) >= n // 3] = 0.0
    amp[np.abs(KZ) >= n // 3] = 0.0
    comps = []
    for _ in range(3):
        ph = rng.uniform(0, 2 * np.pi, (n, n, n))
        comps.append(np.real(np.fft.ifftn(amp * np.exp(1j * ph))) * n ** 3)
    u, v, w = comps
    s = urms / np.sqrt((u ** 2 + v ** 2 + w ** 2).mean() / 3.0)
    u, v, w = (np.asfortranarray(c * s) for c in (u, v, w))
    wE = np.asfortranarray(np.concatenate([w, w[:, :, :1]], axis=2))
    return u, v, wE
