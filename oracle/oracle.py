"""ctypes bindings to the oracle (test infrastructure only).

The oracle is a CPU FP64 restatement of the PadeOps compact operators
(``oracle/padeops_oracle.c``).  Only the tests, ``__graft_entry__.smoke`` and the
CPU-baseline leg of ``bench.py`` may import this module; it is the checker, never
the thing measured or shipped.

Arrays are Fortran-ordered (x fastest), exactly like the reference's
``real(rkind), dimension(n1,n2,n3)`` arguments; ``dir`` 1/2/3 selects the line
direction like the reference's ``dd1/dd2/dd3``.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libpadeops_oracle.so")
_lib = None

STAGG_OPS = {"ddz_E2C": 0, "ddz_C2E": 1, "ddz_C2C": 2, "ddz_E2E": 3,
             "d2dz2_C2C": 4, "d2dz2_E2E": 5, "InterpZ_E2C": 6, "InterpZ_C2E": 7}


def build():
    """Compile the oracle library (gcc; a few seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        _lib = ctypes.CDLL(_LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        i, d = ctypes.c_int, ctypes.c_double
        _lib.oracle_cd06.argtypes = [i, d, i, i, i, i, i, dp, dp, i, i, i]
        _lib.oracle_cd10.argtypes = [i, d, i, i, i, i, i, dp, dp, i, i, i]
        _lib.oracle_cf90.argtypes = [i, i, i, i, i, dp, dp, i, i, i]
        _lib.oracle_gaussian.argtypes = [i, i, i, i, i, dp, dp, i, i, i]
        _lib.oracle_stagg.argtypes = [i, d, i, i, i, i, i, i, i, dp, dp, i, i, i]
        _lib.oracle_threads.argtypes = []
        _lib.oracle_threads.restype = ctypes.c_int
        for fn in ("oracle_cd06", "oracle_cd10", "oracle_cf90", "oracle_gaussian", "oracle_stagg"):
            getattr(_lib, fn).restype = ctypes.c_int
    return _lib


def threads():
    """Host threads the oracle's line loops use (OpenMP)."""
    return lib().oracle_threads()


def _as_f3(f):
    """Return a Fortran-contiguous float64 3-D view plus its shape."""
    f = np.asfortranarray(f, dtype=np.float64)
    if f.ndim == 1:
        f = f.reshape((f.shape[0], 1, 1), order="F")
    elif f.ndim == 2:
        f = f.reshape(f.shape + (1,), order="F")
    return f


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleError(RuntimeError):
    def __init__(self, code):
        super().__init__(f"oracle returned status {code}")
        self.code = code


def _check(rc):
    if rc != 0:
        raise OracleError(rc)


def cd06(f, dx, periodic=True, bc1=0, bcn=0, order=1, dir=1):
    f = _as_f3(f)
    out = np.zeros_like(f, order="F")
    n = f.shape[dir - 1]
    _check(lib().oracle_cd06(n, dx, int(periodic), bc1, bcn, order, dir, _ptr(f), _ptr(out), *f.shape))
    return out


def cd10(f, dx, periodic=True, bc1=0, bcn=0, order=1, dir=1):
    f = _as_f3(f)
    out = np.zeros_like(f, order="F")
    n = f.shape[dir - 1]
    _check(lib().oracle_cd10(n, dx, int(periodic), bc1, bcn, order, dir, _ptr(f), _ptr(out), *f.shape))
    return out


def cf90(f, periodic=True, bc1=0, bcn=0, dir=1):
    f = _as_f3(f)
    out = np.zeros_like(f, order="F")
    n = f.shape[dir - 1]
    _check(lib().oracle_cf90(n, int(periodic), bc1, bcn, dir, _ptr(f), _ptr(out), *f.shape))
    return out


def gaussian(f, periodic=True, bc1=0, bcn=0, dir=1):
    f = _as_f3(f)
    out = np.zeros_like(f, order="F")
    n = f.shape[dir - 1]
    _check(lib().oracle_gaussian(n, int(periodic), bc1, bcn, dir, _ptr(f), _ptr(out), *f.shape))
    return out


def stagg(f, n, dx, op, periodic=True, topEven=False, botEven=False, topSided=False, botSided=False, dir=3):
    """Staggered CD06 operator ``op`` (a name of STAGG_OPS) on cell count ``n``."""
    f = _as_f3(f)
    opi = STAGG_OPS[op]
    out_len = n + 1 if op in ("ddz_C2E", "ddz_E2E", "d2dz2_E2E", "InterpZ_C2E") else n
    shape = list(f.shape)
    shape[dir - 1] = out_len
    out = np.zeros(shape, order="F")
    _check(lib().oracle_stagg(n, dx, int(periodic), int(topEven), int(botEven), int(topSided), int(botSided),
                              opi, dir, _ptr(f), _ptr(out), *f.shape))
    return out
