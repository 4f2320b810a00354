"""The 256-point transform kernels against numpy and the oracle (GPU).

Several double-float kernels run only on 256-point lines: the paired x transforms
(k_fft_df_r2c_pair256, k_fft_df_c2r_pair256: two fields, or a field and its x derivative,
in one launch), the register four-step y transform with its i k and test-filter
multipliers (k_fft_df256<MUL_IK_A / MUL_IK_P / MUL_MASK_AP>), and the fused four-step z
kernel of the projection, the dealiasing and PoissonPeriodic (k_fft_df256_fk).  The 256^3
LES runs on them.  These tests take those branches at shapes the oracle finishes in
seconds: x-y planes of 256 x 256 with a few z planes, and z lines of 256 points under a
small x-y plane.  The same entry points at other sizes take the generic kernels, so each
case is also run at a size where they apply.

Tolerances (normwise relative, each output against its own maximum): transforms 2e-13
(the double-float FFT's ~log2(n) 2^-47); fields after the LES init sequence 1e-12, after
one step 1e-10, the dynamic coefficient 1e-9 (as in test_gpu_les.py); projection and
PoissonPeriodic 1e-12.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import padeops_gb300 as P
from oracle import spectral_oracle as SO
from padeops_gb300 import _lib as L
from padeops_gb300.synthetic import hit_initial_field
from tests.fields import relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FFT_TOL = 2e-13
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()


def host(t):
    return np.asfortranarray(t.cpu().numpy().T)


@pytest.fixture(params=[L.FFT_DF, L.FFT_FP64], ids=["df", "fp64"])
def arith(request, native_lib):
    old = native_lib.pade_fft_get_arith()
    L.check(native_lib.pade_fft_set_arith(request.param))
    yield request.param
    native_lib.pade_fft_set_arith(old)


def _two_fields(nx, ny, nz, seed):
    """Two real fields 1e6 apart in magnitude; the second has an all-zero x line."""
    rng = np.random.default_rng(seed)
    f1 = np.asfortranarray(rng.standard_normal((nx, ny, nz)))
    f2 = np.asfortranarray(1e-6 * rng.standard_normal((nx, ny, nz)))
    f2[:, 3 % ny, nz - 1] = 0.0
    return f1, f2


SHAPES = [(256, 256, 3), (64, 32, 3)]  # the 256-point kernels, then the generic ones


@pytest.mark.parametrize("nx,ny,nz", SHAPES)
@pytest.mark.parametrize("fix", [True, False])
def test_fused_spectral_transforms_match_numpy(native_lib, arith, nx, ny, nz, fix):
    dx, dy = 2 * np.pi / nx, 2 * np.pi / ny
    sp = P.spectral()
    sp.init(nx, ny, nz, dx, dy, fixOddball=fix)
    k1, k2 = SO.spectral_wavenumbers(nx, ny, dx, dy, fix)
    K1, K2 = k1[:, None, None], k2[None, :, None]
    f1, f2 = _two_fields(nx, ny, nz, 17)
    F1, F2 = dev(f1), dev(f2)
    H1 = torch.empty((nz, ny, nx // 2 + 1), dtype=torch.complex128, device="cuda")
    H2 = torch.empty_like(H1)
    # fft of two fields in one pass: each keeps its own relative accuracy
    sp.fft_two(F1, F2, H1, H2)
    torch.cuda.synchronize()
    h1, h2 = SO.fft2_x2y(f1), SO.fft2_x2y(f2)
    assert relerr(host(H1), h1) < FFT_TOL
    assert relerr(host(H2), h2) < FFT_TOL
    keep1, keep2 = H1.clone(), H2.clone()
    o1 = torch.empty_like(F1)
    o2 = torch.empty_like(F1)
    # ifft with the i k1 / i k2 multipliers
    for d, K in ((1, K1), (2, K2)):
        sp.ifft_ik(H2, o1, d)
        torch.cuda.synchronize()
        assert relerr(host(o1), SO.ifft2_y2x(1j * K * h2, nx)) < FFT_TOL, d
    # a field and its x derivative from one pass
    sp.ifft_and_ddx(H2, o1, o2)
    torch.cuda.synchronize()
    assert relerr(host(o1), f2) < FFT_TOL
    assert relerr(host(o2), SO.ifft2_y2x(1j * K1 * h2, nx)) < FFT_TOL
    # two inverse transforms in one pass, with and without multipliers
    for d1, d2 in ((0, 0), (1, 2), (2, 0), (0, 1)):
        sp.ifft_two(H1, d1, H2, d2, o1, o2)
        torch.cuda.synchronize()
        m1 = {0: 1.0, 1: 1j * K1, 2: 1j * K2}[d1]
        m2 = {0: 1.0, 1: 1j * K1, 2: 1j * K2}[d2]
        assert relerr(host(o1), SO.ifft2_y2x(m1 * h1, nx)) < FFT_TOL, (d1, d2)
        assert relerr(host(o2), SO.ifft2_y2x(m2 * h2, nx)) < FFT_TOL, (d1, d2)
    # the sharp test filter fused into the inverse transform
    for filt in (2.0, 1.5):
        sp.ifft_testfilter(H1, o1, filt)
        torch.cuda.synchronize()
        G = ((np.abs(K1) < (2.0 / 3.0) * np.pi / dx / filt) & (np.abs(K2) < (2.0 / 3.0) * np.pi / dy / filt))
        assert relerr(host(o1), SO.ifft2_y2x(G * h1, nx)) < FFT_TOL, filt
    assert torch.equal(H1, keep1) and torch.equal(H2, keep2)  # inputs are not modified
    sp.destroy()


def test_paired_inverse_transform_keeps_each_fields_scale(native_lib):
    """Two half spectra 1e12 apart through one paired x launch (nx = 256), and a spectrum
    whose lines are all zero beside a non-zero one."""
    old = native_lib.pade_fft_get_arith()
    L.check(native_lib.pade_fft_set_arith(L.FFT_DF))
    try:
        nx, ny, nz = 256, 8, 2
        sp = P.spectral()
        sp.init(nx, ny, nz, 2 * np.pi / nx, 2 * np.pi / ny)
        rng = np.random.default_rng(5)
        f1 = np.asfortranarray(1e6 * rng.standard_normal((nx, ny, nz)))
        f2 = np.asfortranarray(1e-6 * rng.standard_normal((nx, ny, nz)))
        h1, h2 = SO.fft2_x2y(f1), SO.fft2_x2y(f2)
        o1 = torch.empty_like(dev(f1))
        o2 = torch.empty_like(o1)
        sp.ifft_two(dev(h1), 0, dev(h2), 0, o1, o2)
        torch.cuda.synchronize()
        assert relerr(host(o1), f1) < FFT_TOL and relerr(host(o2), f2) < FFT_TOL
        z = np.zeros_like(h2)
        sp.ifft_two(dev(h1), 1, dev(z), 2, o1, o2)
        torch.cuda.synchronize()
        assert np.all(host(o2) == 0.0)
        assert relerr(host(o1), SO.ifft2_y2x(1j * SO.spectral_wavenumbers(nx, ny, 2 * np.pi / nx,
                                                                           2 * np.pi / ny)[0][:, None, None] * h1,
                                              nx)) < FFT_TOL
        sp.destroy()
    finally:
        native_lib.pade_fft_set_arith(old)


def _velocity(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    u, v, w = (np.asfortranarray(rng.standard_normal((nx, ny, nz))) for _ in range(3))
    uh, vh, wh = SO.fft2_x2y(u), SO.fft2_x2y(v), SO.fft2_x2y(w)
    whE = np.concatenate([wh, wh[:, :, :1]], axis=2)
    return uh, vh, np.asfortranarray(whE)


@pytest.mark.parametrize("nx,ny,nz", [(8, 8, 256), (16, 4, 256)])
def test_projection_on_256_point_z_lines(native_lib, oracle, arith, nx, ny, nz):
    dx, dy, dz = 2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz
    sp = P.spectral()
    sp.init(nx, ny, nz, dx, dy)
    po = P.padepoisson()
    po.init(dx, dy, dz, sp)
    ref = SO.PeriodicPoisson(nx, ny, nz, dx, dy, dz)
    uh, vh, wh = _velocity(nx, ny, nz, 21)
    U, V, W = dev(uh), dev(vh), dev(wh)
    po.PressureProjection(U, V, W)
    torch.cuda.synchronize()
    ru, rv, rw, _ = ref.projection(uh, vh, wh)
    assert relerr(host(U), ru) < 1e-12
    assert relerr(host(V), rv) < 1e-12
    assert relerr(host(W), rw) < 1e-12
    div = torch.empty((nz, ny, nx), dtype=torch.float64, device="cuda")
    po.DivergenceCheck(U, V, W, div)
    # the divergence sums three derivatives; with 256 z points the staggered z derivative
    # multiplies the velocity's last-bit differences by up to 1/dz, so the error is measured
    # against the largest of the three terms (each at most ~ k_max times its field)
    zc, ze = np.zeros_like(ru), np.zeros_like(rw)
    scale = max(np.abs(ref.divergence(ru, zc, ze)).max(), np.abs(ref.divergence(zc, rv, ze)).max(),
                np.abs(ref.divergence(zc, zc, rw)).max())
    assert np.abs(host(div) - ref.divergence(ru, rv, rw)).max() < 1e-12 * scale
    po.destroy()
    sp.destroy()


def _cd06_modk(kd):
    kd[:] = SO.getmodCD06stagg(kd, 1.0)


@pytest.mark.parametrize("modk", [False, True])
def test_poisson_periodic_on_256_point_z_lines(native_lib, arith, modk):
    nx, ny, nz = 8, 4, 256
    dx, dy, dz = 2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz
    pp = P.PoissonPeriodic()
    cb = (_cd06_modk,) * 3 if modk else ()
    pp.init(dx, dy, dz, nx, ny, nz, 3, *cb)
    rng = np.random.default_rng(13)
    r = np.asfortranarray(rng.standard_normal((nx, ny, nz)))
    R = dev(r)
    F = torch.empty_like(R)
    pp.poisson_solve(R, F)
    torch.cuda.synchronize()
    ref = SO.poisson_periodic(r, dx, dy, dz, cb) if modk else SO.poisson_periodic(r, dx, dy, dz)
    assert relerr(host(F), ref) < 1e-12
    pp.destroy()


# ---------------------------------------------------------------- LES on 256-point lines
LES_FIELDS = ["u", "v", "wC", "w", "uE", "vE"]


def _les_pair(shape, scale=(1.0, 1.0, 1.0), kp=4.0, **kw):
    from oracle.les_oracle import LesOracle

    nx, ny, nz = shape
    L_ = 2 * np.pi
    u, v, w = hit_initial_field(shape, seed=4, kp=kp)
    u, v, w = (np.asfortranarray(a * s) for a, s in zip((u, v, w), scale))
    ref = LesOracle(nx, ny, nz, L_, L_, L_, **kw)
    ref.init_fields(u, v, w)
    g = P.igrid()
    okw = dict(kw)
    if "dynamic" in okw:
        okw["DynamicProcedureType"] = 1 if okw.pop("dynamic") else 0
    g.init(nx, ny, nz, **okw)
    g.set_fields(dev(u), dev(v), dev(w))
    return g, ref


def _les_compare(g, ref, tol):
    for name in LES_FIELDS:
        assert relerr(host(g.field(name)), getattr(ref, name)) < tol, name
    # gradients: a derivative on a fine grid multiplies its field's last-bit differences by
    # up to the grid's largest wavenumber pi/h, so each du_i/dx_j is measured against
    # max|u_i| pi/h_j, the largest derivative the grid can represent
    h = (2 * np.pi / ref.nx, 2 * np.pi / ref.ny, 2 * np.pi / ref.nz)
    vel = {"C": (ref.u, ref.v, ref.wC), "E": (ref.uE, ref.vE, ref.w)}
    for grid, arrs in (("C", ref.duidxjC), ("E", ref.duidxjE)):
        for i in range(9):
            comp, d = i // 3, i % 3  # igrid order: du/dx, du/dy, du/dz, dv/dx, ...
            scale = max(np.abs(arrs[i]).max(), np.abs(vel[grid][comp]).max() * np.pi / h[d])
            err = np.abs(host(g.field(f"duidxj{grid}{i + 1}")) - arrs[i]).max()
            assert err < tol * scale, (grid, i + 1, err / scale)
    for name, arr in (("uhat", ref.uhat), ("vhat", ref.vhat), ("what", ref.what)):
        assert relerr(host(g.field(name)), arr) < tol, name


@pytest.mark.parametrize("shape", [(256, 256, 8), (16, 16, 256)], ids=["xy256", "z256"])
def test_les_step_on_256_point_lines(oracle, shape):
    """xy256 runs the paired x transforms and the y four-step kernels with their
    multipliers; z256 the fused z kernels of the dealiasing and the projection.  The
    spectrum peaks at k = 24 so that the field has energy above the test filter's cutoff
    (k = 42 on the 256-point planes) and the dynamic coefficient is not zero."""
    g, ref = _les_pair(shape, kp=24.0)
    _les_compare(g, ref, 1e-12)
    g.timeAdvance(use_graph=False)
    ref.tvd_rk3()
    _les_compare(g, ref, 1e-10)
    lam = g.info()["lambda"]
    assert np.max(np.abs(ref.lambda1d)) > 1e-9  # not the roundoff of a zero coefficient
    assert np.max(np.abs(lam - ref.lambda1d)) <= 1e-9 * np.max(np.abs(ref.lambda1d))


def test_les_with_disparate_magnitudes_on_256_point_lines(oracle):
    """Velocity components 1e6 apart through the paired x transforms: each field of a pair
    keeps its own scaling, so the small component stays at full relative precision."""
    g, ref = _les_pair((256, 256, 8), scale=(1.0, 1e-6, 1e3))
    _les_compare(g, ref, 1e-12)
    g.timeAdvance(use_graph=False)
    ref.tvd_rk3()
    _les_compare(g, ref, 1e-10)


def test_les_256_without_four_step_kernels_matches_oracle(native_lib):
    """The same step with the four-step and paired kernels switched off (the radix-4
    kernels everywhere), in a fresh process since the switch is read once."""
    env = dict(os.environ, PADE_FFT_FOURSTEP="0")
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-p", "no:cacheprovider",
                        "tests/test_gpu_n256.py::test_les_step_on_256_point_lines"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
