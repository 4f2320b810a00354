"""Mirror of module PoissonPeriodicMod (src/utilities/PoissonPeriodic.F90): type PoissonPeriodic.

Triply periodic FFT Poisson solve lap f = rhs on real (nx, ny, nz) CUDA tensors, with
optional modified-wavenumber callbacks ``Get_ModKx/y/z(kd)`` that map k*d to k'*d in
place (a numpy array), as the reference's procedure arguments do.
"""
import ctypes

import numpy as np

from . import _lib as L
from .spectralMod import _dev


def _wrap(fn):
    if fn is None:
        return L.MODK_FN()

    def cb(ptr, n):
        arr = np.ctypeslib.as_array(ptr, shape=(n,))
        fn(arr)

    return L.MODK_FN(cb)


class PoissonPeriodic:
    def __init__(self):
        self._h = ctypes.c_void_p(None)

    def init(self, dx, dy, dz, nx, ny, nz, dir_id=1, Get_ModKx=None, Get_ModKy=None, Get_ModKz=None):
        """PoissonPeriodic.F90:120-210 (gp's global sizes given directly as nx, ny, nz)."""
        self.destroy()
        h = ctypes.c_void_p(None)
        cbs = [_wrap(f) for f in (Get_ModKx, Get_ModKy, Get_ModKz)]
        L.check(L.lib().pade_poisson3d_init(ctypes.byref(h), int(nx), int(ny), int(nz), float(dx), float(dy),
                                            float(dz), int(dir_id), *cbs), "PoissonPeriodic.init")
        self._h = h

    @property
    def handle(self):
        if not self._h.value:
            raise L.PadeError(L.PADE_EINVAL, "PoissonPeriodic used before init")
        return self._h

    def poisson_solve(self, rhs, f=None):
        """In place (f omitted: rhs is overwritten) or out of place, like the generic."""
        pr, _, s = _dev(rhs, "rhs")
        pf = pr if f is None else _dev(f, "f")[0]
        L.check(L.lib().pade_poisson3d_solve(self.handle, pr, pf, s), "poisson_solve")

    def destroy(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pade_poisson3d_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
