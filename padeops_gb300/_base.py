"""Shared plumbing of the Fortran-API mirror classes.

Each class mirrors one reference Fortran derived type: the same procedure names and
argument meaning; arrays are Fortran-ordered (x fastest) FP64 buffers, given as CUDA
torch tensors (asynchronous on torch's current stream) or host numpy arrays / CPU
tensors (staged through device memory by the library, synchronous).
"""
import ctypes

import numpy as np

from . import _lib as L

try:  # torch is plumbing only: device memory and streams
    import torch
except ImportError:  # pragma: no cover - torch is present in every supported setup
    torch = None


def buffer(a, what, complex_ok=False, dtype=np.float64):
    """Return (pointer, is_complex, stream, nelem_real) of a contiguous array argument."""
    if torch is not None and isinstance(a, torch.Tensor):
        if not a.is_contiguous():
            raise ValueError(f"{what} must be contiguous")
        tdt = {np.float64: torch.float64, np.float32: torch.float32}[dtype]
        cdt = torch.complex128 if dtype == np.float64 else torch.complex64
        if a.dtype == cdt and complex_ok:
            cplx = True
        elif a.dtype == tdt:
            cplx = False
        else:
            raise TypeError(f"{what} has dtype {a.dtype}, expected {tdt}")
        stream = torch.cuda.current_stream(a.device).cuda_stream if a.is_cuda else None
        return a.data_ptr(), cplx, stream, a.numel() * (2 if cplx else 1)
    if isinstance(a, np.ndarray):
        if not (a.flags["F_CONTIGUOUS"] or a.flags["C_CONTIGUOUS"]):
            raise ValueError(f"{what} must be contiguous")
        cdt = np.complex128 if dtype == np.float64 else np.complex64
        if a.dtype == cdt and complex_ok:
            cplx = True
        elif a.dtype == dtype:
            cplx = False
        else:
            raise TypeError(f"{what} has dtype {a.dtype}, expected {np.dtype(dtype)}")
        if not a.flags["WRITEABLE"] and what.startswith("out"):
            raise ValueError(f"{what} is read-only")
        return a.ctypes.data, cplx, None, a.size * (2 if cplx else 1)
    raise TypeError(f"{what} must be a torch.Tensor or numpy.ndarray")


class PadeObject:
    """Owns one library handle (the reference type's allocated LU/penta arrays)."""

    family = None

    def __init__(self):
        self._h = ctypes.c_void_p(None)
        self._path = L.PATH_DF

    @property
    def handle(self):
        if not self._h.value:
            raise L.PadeError(L.PADE_EINVAL, f"{type(self).__name__} used before init")
        return self._h

    def _init(self, fn, *args):
        self.destroy()
        h = ctypes.c_void_p(None)
        rc = fn(ctypes.byref(h), *args)
        if rc == L.PADE_OK:
            self._h = h
            if self._path != L.PATH_DF:
                L.check(L.lib().pade_set_path(self._h, self._path), "set_path")
        return rc

    def destroy(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pade_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def set_path(self, path):
        """Arithmetic path of the FP64 entry points: PATH_DF (default) or PATH_NATIVE."""
        self._path = path
        if self._h.value:
            L.check(L.lib().pade_set_path(self._h, path), "set_path")

    def lengths(self, opcode):
        a, b = ctypes.c_int(), ctypes.c_int()
        L.check(L.lib().pade_get_lengths(self.handle, opcode, ctypes.byref(a), ctypes.byref(b)), "get_lengths")
        return a.value, b.value

    def get_status(self):
        v = ctypes.c_int()
        L.check(L.lib().pade_get_status(self.handle, ctypes.byref(v)), "get_status")
        return v.value

    def apply(self, opcode, dir, f, out, na, nb, bc1=0, bcn=0, path=None):
        """Generic entry (pade_apply): any direction, FP64 or (path=PATH_FP32) FP32 data."""
        path = self._path if path is None else path
        dt = np.float32 if path == L.PATH_FP32 else np.float64
        pf, cf, sf, _ = buffer(f, "f", True, dt)
        po, co, so, _ = buffer(out, "out", True, dt)
        if cf != co:
            raise TypeError("f and out must both be real or both complex")
        stream = sf if sf is not None else so
        L.check(L.lib().pade_apply(self.handle, opcode, dir, int(cf), pf, po, na, nb, bc1, bcn, path, stream),
                f"{type(self).__name__}.apply")

    def _call(self, fn, name, f, out, *ints, complex_fn=None):
        pf, cf, sf, _ = buffer(f, "f", complex_fn is not None)
        po, co, so, _ = buffer(out, "out", complex_fn is not None)
        if cf != co:
            raise TypeError("f and out must both be real or both complex")
        stream = sf if sf is not None else so
        use = complex_fn if cf else fn
        L.check(use(self.handle, pf, po, *ints, stream), f"{type(self).__name__}.{name}")
