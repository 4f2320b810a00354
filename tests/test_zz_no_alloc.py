"""pade_apply_noalloc against pade_apply (GPU).

pade_apply_noalloc serves callers that cannot allocate device memory once their time loop
runs -- a solver that handed the device memory to its own pool at start-up, a process
under a hard device-memory quota, or a multi-stream loop that cannot absorb the device
synchronisation an allocation may cause.  It must give the same results as the regular
entry point, call after call, although every call reuses one static device array, and a
warmed-up call must leave the device's free memory unchanged.

This file is collected last so a run that stops at the first failure has already run every
other test; it passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

from padeops_gb300 import _lib as L
from tests.fields import relerr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

N, NA, NB = 64, 24, 10


def _shape(dir):
    s = [NA, NB]
    s.insert(dir - 1, N)
    return tuple(s)


def _fields(seed, dir, cplx):
    rng = np.random.default_rng(seed)
    shape = _shape(dir)
    x = np.linspace(0, 2 * np.pi, N, endpoint=False)
    bshape = [1, 1, 1]
    bshape[dir - 1] = N
    f = np.sin(3 * x).reshape(bshape) + 0.2 * rng.standard_normal(shape)
    if cplx:
        f = f + 1j * (np.cos(2 * x).reshape(bshape) + 0.2 * rng.standard_normal(shape))
    return np.asfortranarray(f)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def _objects():
    import padeops_gb300 as P

    c = P.cd10()
    assert c.init(N, 2 * np.pi / N, True) == 0
    z = P.cd10()
    assert z.init(N, 1.0 / (N - 1), False) == 0
    return c, z


@pytest.mark.parametrize("cplx", [0, 1], ids=["real", "complex"])
@pytest.mark.parametrize("dir", [1, 2, 3])
def test_noalloc_matches_pade_apply_on_consecutive_calls(native_lib, dir, cplx):
    c, z = _objects()
    lib = native_lib
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):  # two calls in a row: stale contents of the shared array must not leak
        f = _fields(100 + call, dir, cplx)
        for obj, opcode, bc in ((c, 1, (0, 0)), (c, 2, (0, 0)), (z, 1, (1, -1))):
            ref = np.zeros_like(f, order="F")
            got = np.zeros_like(f, order="F")
            # host buffers: staged through the static array
            L.check(lib.pade_apply(obj.handle, opcode, dir, cplx, _ptr(f), _ptr(ref), NA, NB, bc[0], bc[1],
                                   L.PATH_DF, None))
            L.check(lib.pade_apply_noalloc(obj.handle, opcode, dir, cplx, _ptr(f), _ptr(got), NA, NB, bc[0], bc[1],
                                           None))
            assert relerr(got, ref) < 1e-12
            # device buffers: no staging, asynchronous on the stream
            fd = _dev(f)
            od = torch.empty_like(fd)
            L.check(lib.pade_apply_noalloc(obj.handle, opcode, dir, cplx, ctypes.c_void_p(fd.data_ptr()),
                                           ctypes.c_void_p(od.data_ptr()), NA, NB, bc[0], bc[1], s))
            torch.cuda.synchronize()
            assert relerr(od.cpu().numpy().T, ref) < 1e-12
            # device input, host output (and the reverse): one side staged
            got2 = np.zeros_like(f, order="F")
            L.check(lib.pade_apply_noalloc(obj.handle, opcode, dir, cplx, ctypes.c_void_p(fd.data_ptr()),
                                           _ptr(got2), NA, NB, bc[0], bc[1], s))
            assert relerr(got2, ref) < 1e-12
            od.zero_()
            torch.cuda.synchronize()
            L.check(lib.pade_apply_noalloc(obj.handle, opcode, dir, cplx, _ptr(f), ctypes.c_void_p(od.data_ptr()),
                                           NA, NB, bc[0], bc[1], s))
            torch.cuda.synchronize()
            assert relerr(od.cpu().numpy().T, ref) < 1e-12


def test_noalloc_call_leaves_free_device_memory_unchanged(native_lib):
    """After a first call (which may load the module), calls allocate nothing: the device's
    free memory is the same before and after them."""
    c, _ = _objects()
    lib = native_lib
    f = _fields(7, 1, 0)
    fd = _dev(f)
    od = torch.empty_like(fd)
    got = np.zeros_like(f, order="F")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # set-up call (empty array), then one call of each kind to warm up the launch path
    L.check(lib.pade_apply_noalloc(c.handle, 1, 1, 0, None, None, 0, NB, 0, 0, s))
    L.check(lib.pade_apply_noalloc(c.handle, 1, 1, 0, _ptr(f), _ptr(got), NA, NB, 0, 0, None))
    L.check(lib.pade_apply_noalloc(c.handle, 1, 1, 0, ctypes.c_void_p(fd.data_ptr()),
                                   ctypes.c_void_p(od.data_ptr()), NA, NB, 0, 0, s))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        L.check(lib.pade_apply_noalloc(c.handle, 1, 1, 0, _ptr(f), _ptr(got), NA, NB, 0, 0, None))
        L.check(lib.pade_apply_noalloc(c.handle, 1, 1, 0, ctypes.c_void_p(fd.data_ptr()),
                                       ctypes.c_void_p(od.data_ptr()), NA, NB, 0, 0, s))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_buffers_beyond_its_capacity(native_lib):
    import padeops_gb300 as P

    n = 64
    c = P.cd10()
    assert c.init(n, 2 * np.pi / n, True) == 0
    na = L.NOALLOC_SCRATCH_BYTES // (8 * n * 2) + 1  # one host line more than half the array holds
    f = np.zeros((n, na, 1), order="F")
    out = np.zeros_like(f)
    rc = native_lib.pade_apply_noalloc(c.handle, 1, 1, 0, _ptr(f), _ptr(out), na, 1, 0, 0, None)
    assert rc == L.PADE_ESCRATCH
    assert "static staging" in L.strerror(rc)
