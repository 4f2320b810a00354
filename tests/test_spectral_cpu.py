"""Host parts of the spectral / Poisson layer (no GPU): wavenumbers and argument checks."""
import ctypes

import numpy as np
import pytest

from oracle import spectral_oracle as SO
from padeops_gb300 import _lib as L
from padeops_gb300.spectralMod import GetWaveNums, getmodCD06stagg


@pytest.mark.parametrize("n,dx", [(8, 0.25), (64, 2 * np.pi / 64), (7, 0.3), (256, 1.0 / 256), (2, 1.0)])
def test_wavenumbers_match_restatement_bitwise(native_lib, n, dx):
    assert np.array_equal(GetWaveNums(n, dx), SO.GetWaveNums(n, dx))


def test_wavenumbers_known_values(native_lib):
    k = GetWaveNums(8, 2 * np.pi / 8)  # unit box spacing: integer wavenumbers, ifftshifted
    assert np.allclose(k, [0, 1, 2, 3, -4, -3, -2, -1], atol=1e-14)


def test_modified_wavenumber_cd06stagg(native_lib):
    n, dz = 64, 2 * np.pi / 64
    k = GetWaveNums(n, dz)
    kp = getmodCD06stagg(k, dz)
    ref = SO.getmodCD06stagg(k, dz)
    assert np.max(np.abs(kp - ref)) <= 4 * np.finfo(float).eps * np.max(np.abs(ref))
    # sixth-order accurate at small k*dz; exact zero at k = 0; odd in k
    w = np.abs(k * dz)
    small = (w > 0) & (w < 0.3)
    assert np.all(np.abs(kp[small] - k[small]) / np.abs(k[small]) < 0.01 * w[small] ** 6 + 1e-15)
    assert kp[0] == 0.0
    assert np.allclose(kp[1:n // 2], -kp[n - 1:n // 2:-1], rtol=0, atol=1e-13)


def test_init_argument_checks_need_no_gpu(native_lib):
    h = ctypes.c_void_p(None)
    # non power-of-two FFT length is refused before any device work
    assert native_lib.pade_spectral_init(ctypes.byref(h), 12, 16, 8, 0.1, 0.1, 1) == L.PADE_ENOTSUP
    assert native_lib.pade_spectral_init(ctypes.byref(h), 16, 16, 0, 0.1, 0.1, 1) == L.PADE_EINVAL
    cb = L.MODK_FN()
    assert native_lib.pade_poisson3d_init(ctypes.byref(h), 16, 16, 16, 0.1, 0.1, 0.1, 4, cb, cb, cb) == L.PADE_EINVAL
    assert native_lib.pade_poisson3d_init(ctypes.byref(h), 16, 24, 16, 0.1, 0.1, 0.1, 1, cb, cb, cb) == L.PADE_ENOTSUP
    assert native_lib.pade_poisson_periodic_init(ctypes.byref(h), None, 0.1, 0.1, 0.1) == L.PADE_EINVAL
    assert native_lib.pade_transpose(1, 3, None, None, 4, 4, 4, 8, None) == L.PADE_EINVAL
    assert h.value is None


def test_oracle_poisson_manufactured_solution():
    """tests/test_PoissonPeriodic.F90:42-111 on the oracle (Fourier scheme: spectrally exact)."""
    nx, ny, nz = 64, 32, 16
    L_ = 2 * np.pi
    dx, dy, dz = L_ / nx, L_ / ny, L_ / nz
    l, m, n = 6, 3, 1
    x = (np.arange(nx) * dx)[:, None, None]
    y = (np.arange(ny) * dy)[None, :, None]
    z = (np.arange(nz) * dz)[None, None, :]
    ftrue = np.sin(2 * np.pi * l * x / L_) * np.cos(2 * np.pi * m * y / L_) * np.sin(2 * np.pi * n * z / L_)
    rhs = -(l * l + m * m + n * n) * ftrue
    f = SO.poisson_periodic(rhs, dx, dy, dz)
    assert np.max(np.abs(f - ftrue)) < 1e-13


def _wall_velocity(nx, ny, nz, seed, clean=True, wall_w=False):
    from oracle import spectral_oracle as SO

    rng = np.random.default_rng(seed)
    u = rng.standard_normal((nx, ny, nz))
    v = rng.standard_normal((nx, ny, nz))
    w = rng.standard_normal((nx, ny, nz + 1))
    if not wall_w:  # no penetration: w = 0 on both walls
        w[:, :, 0] = 0.0
        w[:, :, nz] = 0.0
    hats = [SO.fft2_x2y(a) for a in (u, v, w)]
    if clean:
        for a in hats:
            a[nx // 2, :, :] = 0.0
            a[:, ny // 2, :] = 0.0
    return hats


@pytest.mark.parametrize("stokes", [False, True])
def test_wall_projection_oracle_properties(oracle, stokes):
    """The restated walled projection (PadePoisson.F90:434-624) leaves the field
    divergence free under the reference's own DivergenceCheck operator (the odd-odd
    staggered ddz_E2C), with w zero on both walls, and is idempotent.  The plain projection
    assumes no penetration on input (its odd extension of w is odd only then); with the
    Stokes-pressure correction a wall-normal velocity on input is removed as well."""
    from oracle import spectral_oracle as SO

    nx, ny, nz = 16, 8, 16
    Lz = 1.0
    wp = SO.WallPoisson(nx, ny, nz, 2 * np.pi / nx, 2 * np.pi / ny, Lz / nz, Lz, stokes=stokes)
    uh, vh, wh = _wall_velocity(nx, ny, nz, 3, wall_w=stokes)
    d0 = np.abs(wp.divergence(uh, vh, wh)).max()
    u2, v2, w2, p = wp.projection(uh, vh, wh)
    assert np.abs(wp.divergence(u2, v2, w2)).max() < 1e-14 * d0
    if not stokes:  # without the correction a wall-normal input velocity leaves divergence
        uw, vw, ww = _wall_velocity(nx, ny, nz, 3, wall_w=True)
        u4, v4, w4, _ = wp.projection(uw, vw, ww)
        assert np.abs(wp.divergence(u4, v4, w4)).max() > 1e-3 * np.abs(wp.divergence(uw, vw, ww)).max()
    assert np.abs(w2[:, :, 0]).max() == 0.0 and np.abs(w2[:, :, nz]).max() == 0.0
    u3, v3, w3, p3 = wp.projection(u2, v2, w2)
    assert max(np.abs(u3 - u2).max(), np.abs(w3 - w2).max()) < 1e-13 * np.abs(uh).max()
