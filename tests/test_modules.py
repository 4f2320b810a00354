"""The per-direction dispatchers: derivatives (derivatives.F90) and filters (filters.F90).

CPU tests cover the method-selection errors, which are raised before any device work;
GPU tests compare every direction of a dispatcher with the oracle on one field.
"""
import numpy as np
import pytest

import padeops_gb300 as P
from padeops_gb300 import _lib as L
from tests.fields import relerr


def test_derivatives_rejects_unknown_and_unprovided_methods():
    d = P.derivatives()
    with pytest.raises(L.PadeError) as e:
        d.init(8, 8, 8, 1.0, 1.0, 1.0, True, True, True, "cd10", "cd07", "cd10")
    assert e.value.code == L.PADE_EINVAL
    for m in ("four", "cheb"):
        with pytest.raises(L.PadeError) as e:
            d.init(8, 8, 8, 1.0, 1.0, 1.0, True, True, True, m, "cd10", "cd10")
        assert e.value.code == L.PADE_ENOTSUP


def test_filters_rejects_lstsq_and_unknown():
    f = P.filters()
    with pytest.raises(L.PadeError) as e:
        f.init(8, 8, 8, True, True, True, "lstsq", "cf90", "cf90")
    assert e.value.code == L.PADE_ENOTSUP
    with pytest.raises(L.PadeError) as e:
        f.init(8, 8, 8, True, True, True, "cf90", "box", "cf90")
    assert e.value.code == L.PADE_EINVAL


def _field(shape, seed):
    rng = np.random.default_rng(seed)
    x = [np.linspace(0, 2 * np.pi, s, endpoint=False) for s in shape]
    X, Y, Z = np.meshgrid(*x, indexing="ij")
    f = np.sin(X + 2 * Y) * np.cos(3 * Z) + 0.05 * rng.standard_normal(shape)
    return np.asfortranarray(f)


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def _host(t):
    return np.asfortranarray(t.cpu().numpy().T)


@pytest.mark.gpu
def test_derivatives_dispatch_matches_oracle(oracle):
    import torch

    nx, ny, nz = 32, 24, 20
    dx, dy, dz = 2 * np.pi / nx, 2 * np.pi / ny, 1.0 / (nz - 1)
    d = P.derivatives()
    d.init(nx, ny, nz, dx, dy, dz, True, True, False, "cd10", "cd06", "cd10")
    assert (d.getMethodx(), d.getMethody(), d.getMethodz()) == (1, 2, 1)
    f = _field((nx, ny, nz), 11)
    fd = _dev(f)
    out = torch.empty_like(fd)
    cases = [
        (d.ddx, {}, oracle.cd10(f, dx, True, order=1, dir=1)),
        (d.d2dx2, {}, oracle.cd10(f, dx, True, order=2, dir=1)),
        (d.ddy, {}, oracle.cd06(f, dy, True, order=1, dir=2)),
        (d.ddz, {}, oracle.cd10(f, dz, False, order=1, dir=3)),
        (d.ddz, {"bc1": 1, "bcn": -1}, oracle.cd10(f, dz, False, 1, -1, order=1, dir=3)),
        (d.d2dz2, {"bc1": -1, "bcn": 1}, oracle.cd10(f, dz, False, -1, 1, order=2, dir=3)),
    ]
    for fn, kw, ref in cases:
        fn(fd, out, **kw)
        torch.cuda.synchronize()
        tol = 1e-12 if fn not in (d.d2dx2, d.d2dz2) else 1e-10
        assert relerr(_host(out), ref) < tol, (fn.__name__, kw)
    with pytest.raises(L.PadeError) as e:  # the reference refuses CD06 second derivatives
        d.d2dy2(fd, out)
    assert e.value.code == 21
    d.destroy()


@pytest.mark.gpu
def test_filters_dispatch_matches_oracle(oracle):
    import torch

    nx, ny, nz = 24, 32, 18
    flt = P.filters()
    flt.init(nx, ny, nz, True, False, False, "cf90", "gaussian", "cf90")
    f = _field((nx, ny, nz), 12)
    fd = _dev(f)
    out = torch.empty_like(fd)
    cases = [
        (flt.filterx, {}, oracle.cf90(f, True, dir=1)),
        (flt.filtery, {"bc1": 1, "bcn": -1}, oracle.gaussian(f, False, 1, -1, dir=2)),
        (flt.filterz, {"bc1": 0, "bcn": 0}, oracle.cf90(f, False, dir=3)),
        (flt.filterz, {"bc1": -1, "bcn": 1}, oracle.cf90(f, False, -1, 1, dir=3)),
    ]
    for fn, kw, ref in cases:
        fn(fd, out, **kw)
        torch.cuda.synchronize()
        assert relerr(_host(out), ref) < 1e-12, (fn.__name__, kw)
    flt.destroy()
