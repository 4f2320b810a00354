"""Host-only helpers around the library's plan-inspection entry points (no GPU)."""
import ctypes

import numpy as np

from padeops_gb300 import _lib as L

STAGG = {name: i for i, name in enumerate(L.STAGG_OPS)}


def params(family, n, dx=1.0, periodic=True, stagg=(False, False, False, False)):
    if family in ("cd06", "cd10"):
        p = [n, dx, int(periodic)]
    elif family in ("cf90", "gaussian"):
        p = [n, int(periodic)]
    else:
        p = [n, dx, int(periodic)] + [int(v) for v in stagg]
    return (ctypes.c_double * len(p))(*p)


def plan_apply_lines(family, prm, opcode, bc1, bcn, lines):
    """Apply the library's host plan to an (nlines, n_in) C-ordered array of lines."""
    lib = L.lib()
    nin, nout = ctypes.c_int(), ctypes.c_int()
    rc = lib.pade_plan_dense(L.FAMILY[family], prm, opcode, bc1, bcn, None, ctypes.byref(nin), ctypes.byref(nout))
    if rc != 0:
        raise L.PadeError(rc, "plan_dense")
    f = np.ascontiguousarray(lines, dtype=np.float64)
    assert f.shape[1] == nin.value
    out = np.zeros((f.shape[0], nout.value))
    dp = ctypes.POINTER(ctypes.c_double)
    L.check(lib.pade_plan_check(L.FAMILY[family], prm, opcode, bc1, bcn, f.ctypes.data_as(dp), out.ctypes.data_as(dp),
                                f.shape[0]), "plan_check")
    return out


def dense(family, prm, opcode, bc1=0, bcn=0):
    lib = L.lib()
    nin, nout = ctypes.c_int(), ctypes.c_int()
    L.check(lib.pade_plan_dense(L.FAMILY[family], prm, opcode, bc1, bcn, None, ctypes.byref(nin), ctypes.byref(nout)))
    M = np.zeros((nout.value, nin.value))
    L.check(lib.pade_plan_dense(L.FAMILY[family], prm, opcode, bc1, bcn,
                                M.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, None))
    return M
