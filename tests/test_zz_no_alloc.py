"""pade_apply_noalloc against pade_apply (GPU).

pade_apply_noalloc serves callers that cannot allocate device memory once their time loop
runs -- a solver that handed the device memory to its own pool at start-up, a process
under a hard device-memory quota, or a multi-stream loop that cannot absorb the device
synchronisation an allocation may cause.  It must give the same results as the regular
entry point, call after call, although every call reuses one static device array.

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


def _fields(seed, shape):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 2 * np.pi, shape[0], endpoint=False)
    f = np.sin(3 * x)[:, None, None] + 0.2 * rng.standard_normal(shape)
    return np.asfortranarray(f)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def test_noalloc_matches_pade_apply_on_consecutive_calls(native_lib):
    import padeops_gb300 as P

    n, na, nb = 64, 24, 10
    dx = 2 * np.pi / n
    c = P.cd10()
    assert c.init(n, dx, True) == 0
    z = P.cd10()
    assert z.init(n, 1.0 / (n - 1), False) == 0
    lib = native_lib
    for call in range(2):  # two calls in a row: stale contents of the shared array must not leak
        f = _fields(100 + call, (n, na, nb))
        for obj, opcode, bc in ((c, 1, (0, 0)), (c, 2, (0, 0)), (z, 1, (1, -1))):
            ref = np.zeros_like(f, order="F")
            got = np.zeros_like(f, order="F")
            # host buffers: staged through the static array
            L.check(lib.pade_apply(obj.handle, opcode, 1, 0, _ptr(f), _ptr(ref), na, nb, bc[0], bc[1], L.PATH_DF, None))
            L.check(lib.pade_apply_noalloc(obj.handle, opcode, 1, 0, _ptr(f), _ptr(got), na, nb, bc[0], bc[1], None))
            assert relerr(got, ref) < 1e-12
            # device buffers: no staging, asynchronous on the stream
            fd = torch.from_numpy(np.ascontiguousarray(f.T)).cuda()
            od = torch.empty_like(fd)
            s = torch.cuda.current_stream().cuda_stream
            L.check(lib.pade_apply_noalloc(obj.handle, opcode, 1, 0, ctypes.c_void_p(fd.data_ptr()),
                                           ctypes.c_void_p(od.data_ptr()), na, nb, bc[0], bc[1], ctypes.c_void_p(s)))
            torch.cuda.synchronize()
            assert relerr(od.cpu().numpy().T, ref) < 1e-12


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
