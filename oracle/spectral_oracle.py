"""numpy restatement of the PadeOps spectral layer and periodic Poisson solvers.

TEST INFRASTRUCTURE ONLY: the tests and the CPU-baseline leg of ``bench.py`` use it as
the checker; the library never calls it.

FFTs are numpy's (pocketfft), standing in for FFTW 3.3.5, which the reference calls with
the same conventions (forward exp(-i..), unnormalised; c2r ignores the imaginary parts of
the mean and Nyquist modes).  The staggered CD06 z derivatives come from the C oracle
(``oracle.stagg``), applied to the real and imaginary parts separately since the
operator coefficients are real.  Arrays are Fortran-shaped numpy arrays indexed (i, j, k).

Parity pinning: GetWaveNums / getmodCD06stagg restate the reference formulas line by line
and the tests compare them bit for bit with the library's host versions; the Poisson solve
is pinned by the reference's manufactured solution (tests/test_PoissonPeriodic.F90:
99-111, Fourier scheme: spectrally exact), the projection by its defining property (the
discrete CD06 divergence vanishes afterwards) and by linear algebra identities.
"""
import numpy as np

from oracle import oracle as C


def GetWaveNums(n, dx):
    """spectral.F90:1748-1764 / PoissonPeriodic.F90:226-242."""
    pi = 4.0 * np.arctan(1.0)
    dummy = n - n % 2
    i = np.arange(1, n + 1, dtype=np.float64)
    k = (-pi + (i - 1) * 2.0 * pi / float(dummy)) / dx
    if n % 2 == 0:
        return np.concatenate([k[n // 2:], k[:n // 2]])
    h = (n + 1) // 2
    return np.concatenate([k[h - 1:], k[:(n - 1) // 2]])


def getmodCD06stagg(k, dz):
    """PadeDerOps.F90:1034-1053."""
    alpha, beta, a, b, c = 9.0 / 62.0, 0.0, 63.0 / 62.0, 17.0 / 62.0, 0.0
    w = np.asarray(k, dtype=np.float64) * dz
    num = 2.0 * a * np.sin(w / 2.0) + (2.0 / 3.0) * b * np.sin(3.0 * w / 2.0) + (2.0 / 5.0) * c * np.sin(5.0 * w / 2.0)
    den = 1.0 + 2.0 * alpha * np.cos(w) + 2.0 * beta * np.cos(2.0 * w)
    return (num / den) / dz


def spectral_wavenumbers(nx, ny, dx, dy, fixOddball=True):
    """k1 (nx/2+1) and k2 (ny) as type spectral stores them (spectral.F90:1025-1075, 1200-1215)."""
    k1 = GetWaveNums(nx, dx)
    k2 = GetWaveNums(ny, dy)
    k1[nx // 2] = -k1[nx // 2]
    k2[ny // 2] = -k2[ny // 2]
    if fixOddball:
        k1[nx // 2] = 0.0
        k2[ny // 2] = 0.0
    return k1[: nx // 2 + 1].copy(), k2


def fft2_x2y(f):
    """fft_3d.F90:645-663: r2c along x, forward c2c along y (unnormalised)."""
    return np.fft.fft(np.fft.rfft(f, axis=0), axis=1)


def ifft2_y2x(fhat, nx, setOddBall=False):
    """fft_3d.F90:616-643: backward c2c y, oddball, c2r x, times 1/(nx ny)."""
    g = np.fft.ifft(fhat, axis=1)  # numpy normalises by 1/ny
    if setOddBall:
        g = g.copy()
        g[nx // 2, :, :] = 0.0
    return np.fft.irfft(g, n=nx, axis=0)  # and by 1/nx


def _stagg_c(f, nz, dz, op):
    return C.stagg(f.real, nz, dz, op, periodic=True) + 1j * C.stagg(f.imag, nz, dz, op, periodic=True)


class PeriodicPoisson:
    """padepoisson with PeriodicInZ (PadePoisson.F90:76-128, 386-432, 1165-1246)."""

    def __init__(self, nx, ny, nz, dx, dy, dz, fixOddball=True):
        self.nx, self.ny, self.nz, self.dz = nx, ny, nz, dz
        self.k1, self.k2 = spectral_wavenumbers(nx, ny, dx, dy, fixOddball)
        k1r = GetWaveNums(nx, dx)[: nx // 2 + 1]
        k2r = GetWaveNums(ny, dy)
        self.k3mod = getmodCD06stagg(GetWaveNums(nz, dz), dz)
        kr = (k1r[:, None, None] ** 2 + k2r[None, :, None] ** 2) + self.k3mod[None, None, :] ** 2
        with np.errstate(divide="ignore"):
            self.kradsq_inv = np.where(kr <= 1e-14, 0.0, 1.0 / kr)

    def projection(self, uhat, vhat, what):
        """PeriodicProjection: returns new (uhat, vhat, what) and the pressure."""
        K1 = self.k1[:, None, None]
        K2 = self.k2[None, :, None]
        f = _stagg_c(what, self.nz, self.dz, "ddz_E2C") + 1j * (K1 * uhat + K2 * vhat)
        F = np.fft.fft(f, axis=2)
        F = -self.kradsq_inv * F
        p = np.fft.ifft(F, axis=2)  # backward transform times 1/nz
        dwE = _stagg_c(p, self.nz, self.dz, "ddz_C2E")
        return uhat - 1j * K1 * p, vhat - 1j * K2 * p, what - dwE, p

    def divergence(self, uhat, vhat, what):
        """DivergenceCheck steps 1-3 (no fixDiv)."""
        K1 = self.k1[:, None, None]
        K2 = self.k2[None, :, None]
        f = _stagg_c(what, self.nz, self.dz, "ddz_E2C") + 1j * K1 * uhat + 1j * K2 * vhat
        return ifft2_y2x(f, self.nx)


def poisson_periodic(rhs, dx, dy, dz, modk=(None, None, None)):
    """PoissonPeriodic.F90:37-111: fft3, times -1/(|k|^2 + 1e-20), zero mode 0, ifft3."""
    nx, ny, nz = rhs.shape
    ks = []
    for n, d, fn in zip((nx, ny, nz), (dx, dy, dz), modk):
        k = GetWaveNums(n, d)
        if fn is not None:
            kd = k * d
            fn(kd)
            k = kd / d
        ks.append(k)
    kx = ks[0][: nx // 2 + 1]
    R = np.fft.fft(np.fft.fft(np.fft.rfft(rhs, axis=0), axis=1), axis=2)
    kabs = ((kx[:, None, None] * kx[:, None, None] + (ks[1] * ks[1])[None, :, None]) + (ks[2] * ks[2])[None, None, :])
    R = R * (-1.0 / (kabs + 1e-20))
    R[0, 0, 0] = 0.0
    return np.fft.irfft(np.fft.ifft(np.fft.ifft(R, axis=2), axis=1), n=nx, axis=0)
