"""The tensor-core dense operator path (3xTF32 on tcgen05) against the oracle (GPU),
along x (contiguous lines) and y, z (strided lines).

Tolerance: 3e-6 normwise relative (max|a-b| / max|b|).  The FP32 accumulation of
256 products bounds the error by ~2^-24 sum|D||f| and the dropped lo*lo term by
~2^-22 |D||f|; sum|D||f| / max|D f| is O(1-10) for these operators and fields.  CF90 runs
in residual form (the tensor cores apply I - D, the epilogue subtracts the result from f in
FP64), so its error scales with the small high-pass part: 3e-7, along every direction.
"""
import ctypes

import numpy as np
import pytest

import padeops_gb300 as P
from padeops_gb300 import _lib as L
from tests.fields import relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def field(n, na, nb, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(n) * 2 * np.pi / n
    f = np.zeros((n, na, nb))
    for _ in range(8):
        k = rng.integers(1, n // 4)
        f += rng.standard_normal() * np.cos(k * x + rng.uniform(0, 6.3))[:, None, None] * \
            rng.standard_normal((1, na, nb))
    return np.asfortranarray(f)


def dense(obj, opcode, f, bc=(0, 0), dir=1):
    na, nb = [s for k, s in enumerate(f.shape) if k != dir - 1]
    fd = torch.from_numpy(np.ascontiguousarray(f.T)).cuda()
    od = torch.full_like(fd, float("nan"))
    lib = L.lib()
    L.check(lib.pade_dense_apply(obj.handle, opcode, dir, ctypes.c_void_p(fd.data_ptr()),
                                 ctypes.c_void_p(od.data_ptr()), na, nb, bc[0], bc[1],
                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    to = ctypes.c_int()
    L.check(lib.pade_dense_status(ctypes.byref(to)))
    assert to.value == 0
    return np.asfortranarray(od.cpu().numpy().T)


@pytest.mark.parametrize("n,na,nb", [(256, 10, 20), (256, 40, 33), (128, 7, 3), (512, 16, 9)])
def test_dense_cd10_periodic(oracle, n, na, nb):
    dx = 2 * np.pi / n
    o = P.cd10()
    assert o.init(n, dx, True) == 0
    f = field(n, na, nb, n + na)
    for order in (1, 2):
        out = dense(o, order, f)
        ref = oracle.cd10(f, dx, periodic=True, order=order, dir=1)
        assert np.isfinite(out).all()
        assert relerr(out, ref) < 3e-6, order


def test_dense_cf90_and_nonperiodic(oracle):
    n, na, nb = 256, 12, 11
    f = field(n, na, nb, 5)
    c = P.cf90()
    assert c.init(n, True) == 0
    assert relerr(dense(c, 0, f), oracle.cf90(f, periodic=True, dir=1)) < 3e-7
    z = P.cd10()
    dz = 1.0 / (n - 1)
    assert z.init(n, dz, False) == 0
    for bc in ((0, 0), (1, -1)):
        out = dense(z, 1, f, bc)
        ref = oracle.cd10(f, dz, periodic=False, bc1=bc[0], bcn=bc[1], order=1, dir=1)
        assert relerr(out, ref) < 3e-6, bc


@pytest.mark.parametrize("dir", [2, 3])
@pytest.mark.parametrize("other", [(40, 9), (128, 3), (7, 130)])
def test_dense_strided_directions(oracle, dir, other):
    n = 256
    dx = 2 * np.pi / n
    o = P.cd10()
    assert o.init(n, dx, True) == 0
    shape = list(other)
    shape.insert(dir - 1, n)
    fx = field(n, other[0], other[1], 7)  # (n, a, b) -> move the operated axis into place
    f = np.asfortranarray(np.moveaxis(fx, 0, dir - 1))
    assert f.shape == tuple(shape)
    for order in (1, 2):
        out = dense(o, order, f, dir=dir)
        ref = oracle.cd10(f, dx, periodic=True, order=order, dir=dir)
        assert np.isfinite(out).all()
        assert relerr(out, ref) < 3e-6, (dir, order)


def test_dense_rejects_unsupported():
    o = P.cd10()
    assert o.init(96, 0.1, True) == 0  # n_out 96 is not a TMEM-friendly size
    f = torch.zeros(96 * 4, dtype=torch.float64, device="cuda")
    g = torch.empty_like(f)
    lib = L.lib()
    rc = lib.pade_dense_apply(o.handle, 1, 1, ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(g.data_ptr()), 4, 1,
                              0, 0, None)
    assert rc == L.PADE_ENOTSUP
    rc = lib.pade_dense_apply(o.handle, 1, 4, ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(g.data_ptr()), 4, 1,
                              0, 0, None)
    assert rc == L.PADE_EINVAL


@pytest.mark.parametrize("dir", [1, 2, 3])
@pytest.mark.parametrize("n,other", [(128, (256, 160)), (256, (128, 200))])
def test_dense_many_tiles_per_cta(dir, n, other):
    # more 128-line tiles than SMs: each CTA of the persistent kernel runs several tiles,
    # so the stage and accumulator hand-offs between tiles are exercised; checked against
    # the double-float line path (itself pinned to the oracle)
    o = P.cd10()
    assert o.init(n, 2 * np.pi / n, True) == 0
    shape = list(other)
    shape.insert(dir - 1, n)
    g = torch.Generator(device="cuda").manual_seed(11 + dir)
    fd = torch.randn(tuple(reversed(shape)), generator=g, dtype=torch.float64, device="cuda")
    na, nb = other
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    lib = L.lib()
    for order in (1, 2):
        od = torch.full_like(fd, float("nan"))
        ref = torch.empty_like(fd)
        L.check(lib.pade_dense_apply(o.handle, order, dir, ctypes.c_void_p(fd.data_ptr()),
                                     ctypes.c_void_p(od.data_ptr()), na, nb, 0, 0, st))
        o.apply(order, dir, fd, ref, na, nb)
        torch.cuda.synchronize()
        to = ctypes.c_int()
        L.check(lib.pade_dense_status(ctypes.byref(to)))
        assert to.value == 0
        assert bool(torch.isfinite(od).all())
        err = float((od - ref).abs().max() / ref.abs().max())
        assert err < 3e-6, (dir, order, err)


@pytest.mark.parametrize("dir,other", [(2, (32, 9)), (3, (16, 4)), (2, (7, 5)), (3, (9, 6))])
def test_dense_cf90_residual_strided(oracle, dir, other):
    """CF90 in residual form along y and z, with (na % 16 == 0) and without the 16-byte
    epilogue stores."""
    n = 256
    c = P.cf90()
    assert c.init(n, True) == 0
    shape = list(other)
    shape.insert(dir - 1, n)
    rng = np.random.default_rng(dir + other[0])
    x = np.arange(n) * 2 * np.pi / n
    prof = np.cos(3 * x) + 0.2 * np.sin(40 * x + 1.0)
    sh = [1, 1, 1]
    sh[dir - 1] = n
    f = np.asfortranarray(prof.reshape(sh) + 0.01 * rng.standard_normal(shape))
    out = dense(c, 0, f, dir=dir)
    assert relerr(out, oracle.cf90(f, periodic=True, dir=dir)) < 3e-7
