"""padepoisson with walls (PeriodicInZ false; PadePoisson.F90:434-624, 320-384, 1165-1246)
against the numpy restatement (GPU).  Tolerance 1e-12 normwise relative, as for the
periodic projection."""
import numpy as np
import pytest

import padeops_gb300 as P
from oracle import spectral_oracle as SO
from padeops_gb300 import _lib as L
from tests.fields import relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()


def host(t):
    return np.asfortranarray(t.cpu().numpy().T)


def _wall_velocity(nx, ny, nz, seed, clean, wall_w=True):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((nx, ny, nz))
    v = rng.standard_normal((nx, ny, nz))
    w = rng.standard_normal((nx, ny, nz + 1))
    if not wall_w:  # no penetration on input
        w[:, :, 0] = 0.0
        w[:, :, nz] = 0.0
    hats = [np.asfortranarray(SO.fft2_x2y(a)) for a in (u, v, w)]
    if clean:
        for a in hats:
            a[nx // 2, :, :] = 0.0
            a[:, ny // 2, :] = 0.0
    return hats


@pytest.fixture(params=[L.FFT_DF, L.FFT_FP64], ids=["df", "fp64"])
def arith(request, native_lib):
    old = native_lib.pade_fft_get_arith()
    L.check(native_lib.pade_fft_set_arith(request.param))
    yield request.param
    native_lib.pade_fft_set_arith(old)


@pytest.mark.parametrize("stokes", [False, True])
@pytest.mark.parametrize("nx,ny,nz", [(16, 8, 16), (32, 16, 32)])
def test_wall_projection_matches_oracle(native_lib, oracle, arith, stokes, nx, ny, nz):
    Lz = 1.3
    dx, dy, dz = 2 * np.pi / nx, 2 * np.pi / ny, Lz / nz
    sp = P.spectral()
    sp.init(nx, ny, nz, dx, dy)
    po = P.padepoisson()
    po.init(dx, dy, dz, sp, PeriodicInZ=False, computeStokesPressure=stokes, Lz=Lz)
    ref = SO.WallPoisson(nx, ny, nz, dx, dy, dz, Lz, stokes=stokes)
    uh, vh, wh = _wall_velocity(nx, ny, nz, 5, clean=False)
    U, V, W = dev(uh), dev(vh), dev(wh)
    po.PressureProjection(U, V, W)
    torch.cuda.synchronize()
    ru, rv, rw, _ = ref.projection(uh, vh, wh)
    assert relerr(host(U), ru) < 1e-12
    assert relerr(host(V), rv) < 1e-12
    assert relerr(host(W), rw) < 1e-12
    assert float(W[0].abs().max()) == 0.0 and float(W[nz].abs().max()) == 0.0
    div = torch.empty((nz, ny, nx), dtype=torch.float64, device="cuda")
    po.DivergenceCheck(U, V, W, div)
    assert relerr(host(div), ref.divergence(ru, rv, rw)) < 1e-12
    # a projected field without oddball modes has no divergence under the odd-odd operator
    # (the plain projection for no-penetration input; the Stokes-pressure correction also
    # removes a wall-normal input velocity)
    uh, vh, wh = _wall_velocity(nx, ny, nz, 7, clean=True, wall_w=stokes)
    d0 = np.abs(ref.divergence(uh, vh, wh)).max()
    U, V, W = dev(uh), dev(vh), dev(wh)
    mx = po.DivergenceCheck(U, V, W, div, fixDiv=True)  # projects: the field is divergent
    assert abs(mx) < 1e-13 * d0
    assert np.abs(host(div)).max() < 1e-13 * d0
    po.destroy()
    sp.destroy()


def test_wall_rejects(native_lib):
    sp = P.spectral()
    sp.init(16, 8, 16, 0.4, 0.8)
    po = P.padepoisson()
    with pytest.raises(L.PadeError) as e:
        po.init(0.4, 0.8, 0.1, sp, PeriodicInZ=False, computeStokesPressure=True, Lz=-1.0)
    assert e.value.code == L.PADE_EINVAL
    po.init(0.4, 0.8, 0.1, sp, PeriodicInZ=False)
    assert po.k3mod is None
    po.destroy()
    sp.destroy()


@pytest.mark.parametrize("walls,stokes", [(False, False), (True, False), (True, True)])
def test_get_pressure_matches_oracle(native_lib, oracle, walls, stokes):
    nx, ny, nz = 16, 8, 16
    Lz = 1.3 if walls else 2 * np.pi
    dx, dy, dz = 2 * np.pi / nx, 2 * np.pi / ny, Lz / nz
    sp = P.spectral()
    sp.init(nx, ny, nz, dx, dy)
    po = P.padepoisson()
    if walls:
        po.init(dx, dy, dz, sp, PeriodicInZ=False, computeStokesPressure=stokes, Lz=Lz)
        ref = SO.WallPoisson(nx, ny, nz, dx, dy, dz, Lz, stokes=stokes)
        uh, vh, wh = _wall_velocity(nx, ny, nz, 11, clean=False)
    else:
        po.init(dx, dy, dz, sp)
        ref = SO.PeriodicPoisson(nx, ny, nz, dx, dy, dz)
        uh, vh, wh = _wall_velocity(nx, ny, nz, 11, clean=False)
        wh = np.asfortranarray(np.concatenate([wh[:, :, :nz], wh[:, :, :1]], axis=2))  # periodic edge plane
    U, V, W = dev(uh), dev(vh), dev(wh)
    pr = torch.empty((nz, ny, nx), dtype=torch.float64, device="cuda")
    po.getPressure(U, V, W, pr)
    torch.cuda.synchronize()
    assert relerr(host(pr), ref.get_pressure(uh, vh, wh)) < 1e-12
    assert relerr(host(U), uh) == 0.0 and relerr(host(W), wh) == 0.0  # inputs unchanged
    pr2 = torch.empty_like(pr)
    po.getPressureAndUpdateRHS(U, V, W, pr2)
    torch.cuda.synchronize()
    assert relerr(host(pr2), host(pr)) < 1e-14
    ru, rv, rw, _ = ref.projection(uh, vh, wh)
    assert relerr(host(U), ru) < 1e-12 and relerr(host(W), rw) < 1e-12
    po.destroy()
    sp.destroy()
