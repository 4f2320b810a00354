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

    def get_pressure(self, uhat, vhat, what):
        """Periodic_getPressure (PadePoisson.F90:716-750): the projection's pressure, physical."""
        return ifft2_y2x(self.projection(uhat, vhat, what)[3], self.nx)


def _stagg_oo(f, nz, dz, op):
    """Pade6stagg ddz with bot = top = -1 on a non-periodic grid: the odd-odd cd06stagg
    (PadeDerOps.F90:92-95, 592-595), real and imaginary parts separately."""
    kw = dict(periodic=False, topEven=False, botEven=False, topSided=False, botSided=False)
    return C.stagg(f.real, nz, dz, op, **kw) + 1j * C.stagg(f.imag, nz, dz, op, **kw)


class WallPoisson:
    """padepoisson with PeriodicInZ false: walls at z = 0 and Lz (PadePoisson.F90:130-318
    init, 434-624 PressureProjection, 320-384 ProjectStokesPressure, 1165-1246
    DivergenceCheck with derivZ%ddz_E2C(.., -1, -1)).  The projection works on the even
    extension of the divergence and the odd extension of w to 2 nz points along z, with the
    CD06-stagg modified wavenumbers phase-shifted by -+ dz/2 (edge <-> centre)."""

    def __init__(self, nx, ny, nz, dx, dy, dz, Lz, stokes=False, fixOddball=True):
        self.nx, self.ny, self.nz, self.dz, self.stokes = nx, ny, nz, dz, stokes
        self.k1, self.k2 = spectral_wavenumbers(nx, ny, dx, dy, fixOddball)  # sp%k1, sp%k2
        self.k1r = GetWaveNums(nx, dx)[: nx // 2 + 1]                       # k1inZ
        self.k2r = GetWaveNums(ny, dy)
        nze = 2 * nz
        k3 = GetWaveNums(nze, dz)
        k3mod = getmodCD06stagg(k3, dz)
        self.k3mc = k3mod * np.exp(1j * (-dz / 2.0) * k3)  # init 194-199
        self.k3mp = k3mod * np.exp(1j * (dz / 2.0) * k3)
        kr = (self.k1r[:, None, None] ** 2 + self.k2r[None, :, None] ** 2) + k3mod[None, None, :] ** 2
        with np.errstate(divide="ignore"):
            self.kinv = np.where(kr <= 1e-14, 0.0, 1.0 / kr)
        if stokes:  # init 235-306
            lam = np.sqrt(self.k1r[:, None] ** 2 + self.k2r[None, :] ** 2)
            temp = lam * Lz
            with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
                den = np.where(temp < 500.0, 1.0 / (lam * np.sinh(np.minimum(temp, 500.0)) + 1e-13), 0.0)
            den[den < 1e-16] = 0.0
            den[0, 0] = 0.0
            self.denFact = den
            zE = np.linspace(0.0, Lz, nz + 1)
            zC = 0.5 * (zE[:-1] + zE[1:])
            L3 = lam[:, :, None]
            t = L3 * (Lz - zC)[None, None, :]
            self.cosh_bot = np.where(t < 32.0, np.cosh(np.minimum(t, 32.0)), 4e13)
            t = L3 * zC[None, None, :]
            self.cosh_top = np.where(t < 32.0, np.cosh(np.minimum(t, 32.0)), 1e13)
            t = L3 * (Lz - zE)[None, None, :]
            self.sinh_bot = np.where(t < 32.0, -L3 * np.sinh(np.minimum(t, 32.0)), -4e13)
            t = L3 * zE[None, None, :]
            self.sinh_top = np.where(t < 32.0, L3 * np.sinh(np.minimum(t, 32.0)), 4e13)

    def projection(self, uhat, vhat, what):
        """PressureProjection: returns new (uhat, vhat, what) and the pressure."""
        nz = self.nz
        u, v, w = uhat.copy(), vhat.copy(), what.copy()
        self.phat_stokes = None
        if self.stokes:
            K1, K2 = self.k1r[:, None, None], self.k2r[None, :, None]
            chat = -w[:, :, 0] * self.denFact  # bottom (ProjectStokesPressure 331-357)
            ph = 1j * chat[:, :, None] * self.cosh_bot
            self.phat_stokes = ph
            u -= K1 * ph
            v -= K2 * ph
            w[:, :, 0] = 0.0
            w[:, :, 1:] -= chat[:, :, None] * self.sinh_bot[:, :, 1:]
            chat = w[:, :, nz] * self.denFact  # top (361-381)
            ph = 1j * chat[:, :, None] * self.cosh_top
            self.phat_stokes = (self.phat_stokes, ph)
            u -= K1 * ph
            v -= K2 * ph
            w[:, :, :nz] -= chat[:, :, None] * self.sinh_top[:, :, :nz]
            w[:, :, nz] = 0.0
        else:
            K1, K2 = self.k1[:, None, None], self.k2[None, :, None]
        f2d = 1j * (K1 * u + K2 * v)
        fext = np.concatenate([f2d[:, :, ::-1], f2d], axis=2)           # step 3 (476-492)
        wext = np.concatenate([-w[:, :, nz - 1:0:-1], w], axis=2)        # (494-510)
        F = np.fft.fft(fext, axis=2)
        W = np.fft.fft(wext, axis=2)
        F = F + 1j * self.k3mc[None, None, :] * W                        # step 5 (518-526)
        F = -F * self.kinv
        W = W - 1j * self.k3mp[None, None, :] * F                        # step 6 (529-536)
        F = np.fft.ifft(F, axis=2)                                       # step 7, times 1/(2 nz)
        W = np.fft.ifft(W, axis=2)
        p = F[:, :, nz:]
        wn = W[:, :, nz - 1:].copy()
        wn[:, :, 0] = 0.0
        wn[:, :, nz] = 0.0
        return u - 1j * K1 * p, v - 1j * K2 * p, wn, p

    def get_pressure(self, uhat, vhat, what):
        """getPressure (PadePoisson.F90:752-898): the projection's pressure plus, with the
        Stokes pressure, phat_z1 + phat_z2 of the same fields; physical."""
        p = self.projection(uhat, vhat, what)[3]
        if self.stokes:
            p = (p + self.phat_stokes[0]) + self.phat_stokes[1]
        return ifft2_y2x(p, self.nx)

    def divergence(self, uhat, vhat, what):
        """DivergenceCheck steps 1-3 (no fixDiv): odd-odd staggered dw/dz + i k1 u + i k2 v."""
        K1 = self.k1[:, None, None]
        K2 = self.k2[None, :, None]
        f = _stagg_oo(what, self.nz, self.dz, "ddz_E2C") + 1j * K1 * uhat + 1j * K2 * vhat
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


def fourier_coll(op, f, nz, dz):
    """Pade6stagg's fourierColl scheme: the spectral layer's periodic-z operators
    (spectral.F90:365-700, factors from its init 843-856).  op in Pade6stagg order (0 ddz_C2E,
    1 ddz_E2C, 2 interpz_C2E, 3 interpz_E2C, 4 d2dz2_C2C, 5 d2dz2_E2E); f Fortran-shaped with z
    last (nz cells or nz + 1 edges, of which the first nz planes are transformed).  Real input:
    r2c, modes 0 .. nz/2 - 1 multiplied (the Nyquist mode passes), c2r; complex input: c2c,
    every mode multiplied; edge outputs repeat plane 0 as plane nz."""
    k = GetWaveNums(nz, dz)
    em, ep = np.exp(-1j * k * dz / 2.0), np.exp(1j * k * dz / 2.0)
    fac = {0: 1j * k * em, 1: 1j * k * ep, 2: em, 3: ep, 4: -(k ** 2), 5: -(k ** 2)}[op]
    x = np.asarray(f)[..., :nz]
    if np.iscomplexobj(x):
        out = np.fft.ifft(np.fft.fft(x, axis=-1) * fac, axis=-1)
    else:
        X = np.fft.rfft(x, axis=-1)
        X[..., :nz // 2] *= fac[:nz // 2]
        out = np.fft.irfft(X, n=nz, axis=-1)
    if op in (0, 2, 5):
        out = np.concatenate([out, out[..., :1]], axis=-1)
    return out
