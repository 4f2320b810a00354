"""FFT layer, spectral transforms, periodic projection, divergence check, PoissonPeriodic and
pencil transposes against the numpy/C oracle (GPU).

Tolerances (normwise relative): FFTs 1e-13 of the output's maximum (radix-2 FFT error
grows like eps*log2(n)); projection and divergence 1e-12, the staggered CD06 operators'
FP64 tolerance.  The manufactured Poisson solution of the reference's own test is checked
against the exact answer at 1e-12 absolute.
"""
import ctypes

import numpy as np
import pytest

import padeops_gb300 as P
from oracle import spectral_oracle as SO
from padeops_gb300 import _lib as L
from tests.fields import relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    """Fortran-ordered numpy array -> CUDA tensor with the same memory layout (reversed dims)."""
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()


def host(t):
    return np.asfortranarray(t.cpu().numpy().T)


def vp(t):
    return ctypes.c_void_p(t.data_ptr())


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def crand(rng, shape):
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


# FFT arithmetic: double-float (default; ~48 bits, error ~log2(n) 2^-47) or native FP64
FFT_TOL = {L.FFT_DF: 2e-13, L.FFT_FP64: 1e-13}


@pytest.fixture(params=[L.FFT_DF, L.FFT_FP64], ids=["df", "fp64"])
def arith(request, native_lib):
    old = native_lib.pade_fft_get_arith()
    L.check(native_lib.pade_fft_set_arith(request.param))
    yield request.param
    native_lib.pade_fft_set_arith(old)


@pytest.mark.parametrize("dir", [1, 2, 3])
@pytest.mark.parametrize("n", [2, 4, 32, 128, 256, 1024, 2048, 8192])
@pytest.mark.parametrize("sign", [-1, 1])
def test_c2c_matches_numpy(native_lib, arith, dir, n, sign):
    tol = FFT_TOL[arith]
    rng = np.random.default_rng(n + dir)
    shape = [5, 3, 7]
    shape[dir - 1] = n
    a = crand(rng, shape)
    x = dev(a)
    y = torch.empty_like(x)
    L.check(native_lib.pade_fft_c2c(dir, sign, vp(x), vp(y), *shape, 0.5, stream()))
    torch.cuda.synchronize()
    ref = 0.5 * (np.fft.fft(a, axis=dir - 1) if sign < 0 else n * np.fft.ifft(a, axis=dir - 1))
    assert relerr(host(y), ref) < tol
    # in place
    L.check(native_lib.pade_fft_c2c(dir, sign, vp(x), vp(x), *shape, 0.5, stream()))
    torch.cuda.synchronize()
    assert relerr(host(x), ref) < tol


@pytest.mark.parametrize("nx", [2, 8, 64, 512, 4096])
def test_r2c_c2r_x(native_lib, arith, nx):
    tol = FFT_TOL[arith]
    rng = np.random.default_rng(nx)
    shape = (nx, 6, 5)
    f = np.asfortranarray(rng.standard_normal(shape))
    x = dev(f)
    h = torch.empty((5, 6, nx // 2 + 1), dtype=torch.complex128, device="cuda")
    L.check(native_lib.pade_fft_r2c_x(vp(x), vp(h), *shape, stream()))
    torch.cuda.synchronize()
    ref = np.fft.rfft(f, axis=0)
    assert relerr(host(h), ref) < tol
    back = torch.empty_like(x)
    L.check(native_lib.pade_fft_c2r_x(vp(h), vp(back), *shape, 1.0 / nx, stream()))
    torch.cuda.synchronize()
    assert relerr(host(back), f) < tol
    # c2r ignores the imaginary parts of the mean and Nyquist entries (like FFTW)
    hh = host(h).copy()
    hh[0] += 3j
    hh[nx // 2] += 5j
    h2 = dev(hh)
    L.check(native_lib.pade_fft_c2r_x(vp(h2), vp(back), *shape, 1.0 / nx, stream()))
    torch.cuda.synchronize()
    assert relerr(host(back), f) < tol


@pytest.mark.parametrize("fix", [True, False])
def test_spectral_fft_ifft(native_lib, arith, fix):
    tol = FFT_TOL[arith]
    nx, ny, nz = 64, 32, 6
    dx, dy = 2 * np.pi / nx, 2 * np.pi / ny
    sp = P.spectral()
    sp.init(nx, ny, nz, dx, dy, fixOddball=fix)
    k1, k2 = SO.spectral_wavenumbers(nx, ny, dx, dy, fix)
    assert np.array_equal(sp.k1_1d, k1) and np.array_equal(sp.k2_1d, k2)
    rng = np.random.default_rng(3)
    f = np.asfortranarray(rng.standard_normal((nx, ny, nz)))
    fd = dev(f)
    fh = torch.empty((nz, ny, nx // 2 + 1), dtype=torch.complex128, device="cuda")
    sp.fft(fd, fh)
    torch.cuda.synchronize()
    ref = SO.fft2_x2y(f)
    assert relerr(host(fh), ref) < tol
    keep = fh.clone()
    out = torch.empty_like(fd)
    for odd in (False, True):
        sp.ifft(fh, out, setOddball=odd)
        torch.cuda.synchronize()
        assert torch.equal(fh, keep)  # the input is not modified
        assert relerr(host(out), SO.ifft2_y2x(ref, nx, odd)) < tol
    sp.destroy()


def _velocity(nx, ny, nz, seed, clean=False):
    """Spectral velocity of a random physical field; w on the nz+1 edges (periodic copy).

    clean removes the x- and y-Nyquist (oddball) modes, as the solver's dealiasing does.
    With fixOddball (the reference default) the projection uses k1 = k2 = 0 there for the
    divergence and the velocity update but the full k1^2 + k2^2 in |k|^2 (PadePoisson.F90:
    94-111 vs spectral.F90:1200-1215), so those modes keep their divergence by design."""
    rng = np.random.default_rng(seed)
    u, v, w = (np.asfortranarray(rng.standard_normal((nx, ny, nz))) for _ in range(3))
    uh, vh, wh = SO.fft2_x2y(u), SO.fft2_x2y(v), SO.fft2_x2y(w)
    if clean:
        for a in (uh, vh, wh):
            a[nx // 2, :, :] = 0.0
            a[:, ny // 2, :] = 0.0
    whE = np.concatenate([wh, wh[:, :, :1]], axis=2)
    return uh, vh, np.asfortranarray(whE)


@pytest.mark.parametrize("nx,ny,nz", [(32, 16, 16), (64, 32, 32), (16, 16, 64)])
def test_pressure_projection_matches_oracle(native_lib, oracle, arith, nx, ny, nz):
    dx, dy, dz = 2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz
    sp = P.spectral()
    sp.init(nx, ny, nz, dx, dy)
    po = P.padepoisson()
    po.init(dx, dy, dz, sp)
    ref = SO.PeriodicPoisson(nx, ny, nz, dx, dy, dz)
    assert np.max(np.abs(po.k3mod - ref.k3mod)) <= 4 * np.finfo(float).eps * np.max(np.abs(ref.k3mod))
    uh, vh, wh = _velocity(nx, ny, nz, 5)
    U, V, W = dev(uh), dev(vh), dev(wh)
    po.PressureProjection(U, V, W)
    torch.cuda.synchronize()
    ru, rv, rw, _ = ref.projection(uh, vh, wh)
    assert relerr(host(U), ru) < 1e-12
    assert relerr(host(V), rv) < 1e-12
    assert relerr(host(W), rw) < 1e-12
    div = torch.empty((nz, ny, nx), dtype=torch.float64, device="cuda")
    mx = po.DivergenceCheck(U, V, W, div)
    assert relerr(host(div), ref.divergence(ru, rv, rw)) < 1e-12
    assert mx == float(host(div).max())
    # the CD06 divergence of a projected field without oddball modes vanishes
    uh, vh, wh = _velocity(nx, ny, nz, 7, clean=True)
    U, V, W = dev(uh), dev(vh), dev(wh)
    d0 = ref.divergence(uh, vh, wh)
    po.PressureProjection(U, V, W)
    po.DivergenceCheck(U, V, W, div)
    assert np.max(np.abs(host(div))) < 1e-13 * np.max(np.abs(d0))
    po.destroy()
    sp.destroy()


def test_divergence_check_and_fixdiv(native_lib, oracle, arith):
    nx, ny, nz = 32, 32, 16
    dx, dy, dz = 2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz
    sp = P.spectral()
    sp.init(nx, ny, nz, dx, dy)
    po = P.padepoisson()
    po.init(dx, dy, dz, sp)
    ref = SO.PeriodicPoisson(nx, ny, nz, dx, dy, dz)
    uh, vh, wh = _velocity(nx, ny, nz, 6, clean=True)
    U, V, W = dev(uh), dev(vh), dev(wh)
    div = torch.empty((nz, ny, nx), dtype=torch.float64, device="cuda")
    mx = po.DivergenceCheck(U, V, W, div)
    d0 = ref.divergence(uh, vh, wh)
    assert relerr(host(div), d0) < 1e-12
    assert mx == pytest.approx(d0.max(), rel=1e-12)
    assert relerr(host(U), uh) == 0.0  # without fixDiv nothing is modified
    # fixDiv: the divergent field is projected, the returned maximum is the re-checked one
    mx2 = po.DivergenceCheck(U, V, W, div, fixDiv=True)
    ru, rv, rw, _ = ref.projection(uh, vh, wh)
    assert relerr(host(U), ru) < 1e-12 and relerr(host(W), rw) < 1e-12
    assert abs(mx2) < 1e-13 * np.abs(d0).max()
    po.destroy()
    sp.destroy()


def _cd06_modk(kd):
    kd[:] = SO.getmodCD06stagg(kd, 1.0)


@pytest.mark.parametrize("dir_id", [1, 3])
def test_poisson_periodic_manufactured(native_lib, arith, dir_id):
    """tests/test_PoissonPeriodic.F90:42-111 (nx, ny, nz = 64, 32, 16; waves 6, 3, 1)."""
    nx, ny, nz = 64, 32, 16
    L_ = 2 * np.pi
    dx, dy, dz = L_ / nx, L_ / ny, L_ / nz
    l, m, n = 6, 3, 1
    x = (np.arange(nx) * dx)[:, None, None]
    y = (np.arange(ny) * dy)[None, :, None]
    z = (np.arange(nz) * dz)[None, None, :]
    ftrue = np.sin(2 * np.pi * l * x / L_) * np.cos(2 * np.pi * m * y / L_) * np.sin(2 * np.pi * n * z / L_)
    rhs = np.asfortranarray(-(4 * np.pi ** 2 * np.cos(2 * np.pi * m * y / L_) * np.sin(2 * np.pi * l * x / L_)
                              * np.sin(2 * np.pi * n * z / L_) * (L_ ** 2 * L_ ** 2 * n ** 2 + L_ ** 2 * L_ ** 2 * m ** 2
                                                                   + L_ ** 2 * L_ ** 2 * l ** 2)) / (L_ ** 6))
    pp = P.PoissonPeriodic()
    pp.init(dx, dy, dz, nx, ny, nz, dir_id)
    R = dev(rhs)
    F = torch.empty_like(R)
    pp.poisson_solve(R, F)
    torch.cuda.synchronize()
    assert np.max(np.abs(host(F) - ftrue)) < 1e-12
    assert relerr(host(F), SO.poisson_periodic(rhs, dx, dy, dz)) < 1e-12
    pp.poisson_solve(R)  # in place
    torch.cuda.synchronize()
    assert np.max(np.abs(host(R) - ftrue)) < 1e-12
    # modified wavenumbers through the callbacks (GetKmod_CD06_stagg of the same test)
    pp.init(dx, dy, dz, nx, ny, nz, dir_id, _cd06_modk, _cd06_modk, _cd06_modk)
    rng = np.random.default_rng(9)
    r = np.asfortranarray(rng.standard_normal((nx, ny, nz)))
    R = dev(r)
    pp.poisson_solve(R, F)
    torch.cuda.synchronize()
    ref = SO.poisson_periodic(r, dx, dy, dz, (_cd06_modk,) * 3)
    assert relerr(host(F), ref) < 1e-12
    pp.destroy()


def test_transposes_are_layout_preserving_copies(native_lib):
    from padeops_gb300 import decomp_2d as D

    rng = np.random.default_rng(1)
    a = dev(np.asfortranarray(rng.standard_normal((8, 6, 4))))
    b = torch.empty_like(a)
    for fn in (D.transpose_x_to_y, D.transpose_y_to_z, D.transpose_z_to_y, D.transpose_y_to_x):
        b.zero_()
        fn(a, b)
        torch.cuda.synchronize()
        assert torch.equal(a, b)
    c = dev(crand(rng, (5, 4, 3)))
    d = torch.empty_like(c)
    D.transpose_y_to_z(c, d)
    torch.cuda.synchronize()
    assert torch.equal(c, d)


@pytest.mark.parametrize("amp", [1e-200, 1e-30, 1.0, 1e30, 1e200])
def test_df_fft_is_scale_invariant(native_lib, amp):
    """The double-float transform scales each line by a power of two, so its relative
    accuracy does not depend on the amplitude (FP64 range, not the float range)."""
    old = native_lib.pade_fft_get_arith()
    L.check(native_lib.pade_fft_set_arith(L.FFT_DF))
    try:
        rng = np.random.default_rng(11)
        shape = [64, 8, 4]
        a = crand(rng, shape) * amp
        a[:, 0, 0] *= 1e-40  # one line far below the others: still accurate relative to itself
        x = dev(a)
        y = torch.empty_like(x)
        for dir in (1, 2, 3):
            sh = list(shape)
            L.check(native_lib.pade_fft_c2c(dir, -1, vp(x), vp(y), *sh, 1.0, stream()))
            torch.cuda.synchronize()
            ref = np.fft.fft(a, axis=dir - 1)
            assert relerr(host(y), ref) < 2e-13, dir
        # the x line scaled by 1e-40 keeps its own relative accuracy
        L.check(native_lib.pade_fft_c2c(1, -1, vp(x), vp(y), *shape, 1.0, stream()))
        torch.cuda.synchronize()
        assert relerr(host(y)[:, 0, 0], np.fft.fft(a[:, 0, 0])) < 2e-13
    finally:
        native_lib.pade_fft_set_arith(old)
