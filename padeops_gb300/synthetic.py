"""Seeded synthetic fields with the shapes and spectra of the benchmark configurations.

The reference's input data (HIT restart files, DNS fields) are not available; these
generators stand in for them.  Arrays are Fortran-ordered (x fastest), like the
reference's fields.
"""
import numpy as np


def random_modes(n, nmodes, kmax, seed, z_nonperiodic=False, profile=False, gradient=False):
    """Sum of nmodes Fourier modes with integer wavevectors |k_i| <= kmax, amplitudes
    N(0,1)*|k|^(-5/6) and random phases on [0, 2pi)^3 (z on [0, 1] when z_nonperiodic,
    times tanh(4(z - 0.5)) when profile).  gradient (periodic, no profile) also returns
    the analytic derivatives (df/dx, df/dy, df/dz)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    x = np.arange(nx) * 2 * np.pi / nx
    y = np.arange(ny) * 2 * np.pi / ny
    if z_nonperiodic:
        zz = np.linspace(0.0, 1.0, nz)
        z = 2 * np.pi * zz
    else:
        z = np.arange(nz) * 2 * np.pi / nz
    if gradient and (z_nonperiodic or profile):
        raise ValueError("analytic gradients of the periodic field only")
    f = np.zeros((nx, ny, nz), order="F")
    grad = [np.zeros((nx, ny, nz), order="F") for _ in range(3)] if gradient else None
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    for _ in range(nmodes):
        k = np.zeros(3)
        while not np.any(k):
            k = rng.integers(-kmax, kmax + 1, size=3)
        amp = rng.standard_normal() * np.linalg.norm(k) ** (-5.0 / 6.0)
        ph = rng.uniform(0, 2 * np.pi)
        arg = k[0] * X + k[1] * Y + k[2] * Z + ph
        f += amp * np.cos(arg)
        if gradient:
            s = np.sin(arg)
            for i in range(3):
                grad[i] -= amp * k[i] * s
    if profile:
        f *= np.tanh(4 * (np.linspace(0.0, 1.0, nz) - 0.5))[None, None, :]
    if gradient:
        return np.asfortranarray(f), [np.asfortranarray(g) for g in grad]
    return np.asfortranarray(f)


def hit_initial_field(n, seed=4, kp=4.0, urms=1.0):
    """Seeded solenoidal-spectrum field on [0, 2pi)^3: E(k) ~ k^4 exp(-2 (k/kp)^2), random
    phases, scaled to u_rms; w returned on nz+1 edge planes (plane nz+1 = plane 1).  The
    projection inside init_fields makes it discretely divergence free.  n is the points
    per direction, or (nx, ny, nz) for a box of unequal resolutions."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    KX, KY, KZ = np.meshgrid(np.fft.fftfreq(nx, 1.0 / nx), np.fft.fftfreq(ny, 1.0 / ny),
                             np.fft.fftfreq(nz, 1.0 / nz), indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    kk[0, 0, 0] = 1.0
    E = kk ** 4 * np.exp(-2.0 * (kk / kp) ** 2)
    amp = np.sqrt(E / (4 * np.pi * kk ** 2))
    amp[0, 0, 0] = 0.0
    amp[np.abs(KX) >= nx // 3] = 0.0
    amp[np.abs(KY) >= ny // 3] = 0.0
    amp[np.abs(KZ) >= nz // 3] = 0.0
    comps = []
    for _ in range(3):
        ph = rng.uniform(0, 2 * np.pi, (nx, ny, nz))
        comps.append(np.real(np.fft.ifftn(amp * np.exp(1j * ph))) * (nx * ny * nz))
    u, v, w = comps
    s = urms / np.sqrt((u ** 2 + v ** 2 + w ** 2).mean() / 3.0)
    u, v, w = (np.asfortranarray(c * s) for c in (u, v, w))
    wE = np.asfortranarray(np.concatenate([w, w[:, :, :1]], axis=2))
    return u, v, wE


def hit_initial_field_torch(n, seed=4, kp=4.0, urms=1.0, device="cuda"):
    """hit_initial_field built on the device (torch FFTs; independent phases from a seeded
    torch generator, so not the same realisation as the numpy version): u, v (nz, ny, nx)
    and w on nz+1 edge planes, as CUDA tensors holding Fortran-ordered arrays (x fastest).
    For grids whose numpy construction would be slow (512^3)."""
    import torch

    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    g = torch.Generator(device=device).manual_seed(seed)
    f = lambda m: torch.fft.fftfreq(m, 1.0 / m, device=device, dtype=torch.float64)  # noqa: E731
    kx, ky, kz = f(nx), f(ny), f(nz)
    # (z, y, x) tensor order = Fortran (x, y, z) memory order
    KZ, KY, KX = kz[:, None, None], ky[None, :, None], kx[None, None, :]
    kk = torch.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    kk[0, 0, 0] = 1.0
    amp = torch.sqrt(kk ** 4 * torch.exp(-2.0 * (kk / kp) ** 2) / (4 * np.pi * kk ** 2))
    amp[0, 0, 0] = 0.0
    amp = amp * (KX.abs() < nx // 3) * (KY.abs() < ny // 3) * (KZ.abs() < nz // 3)
    del kk
    comps = []
    for _ in range(3):
        ph = torch.rand((nz, ny, nx), generator=g, device=device, dtype=torch.float64) * (2 * np.pi)
        comps.append(torch.fft.ifftn(torch.polar(amp, ph)).real.contiguous() * float(nx * ny * nz))
        del ph
    u, v, w = comps
    s = urms / torch.sqrt((u ** 2 + v ** 2 + w ** 2).mean() / 3.0)
    u, v, w = u * s, v * s, w * s
    wE = torch.cat([w, w[:1]], dim=0).contiguous()
    return u.contiguous(), v.contiguous(), wE
