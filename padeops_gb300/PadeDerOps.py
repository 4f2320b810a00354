"""Mirror of module PadeDerOps (src/incompressible/PadeDerOps.F90): type Pade6stagg.

igrid's z-operator facade over the staggered operators.  Scheme cd06: periodic objects use
one periodic cd06stagg; non-periodic objects select one of nine cd06stagg objects per call
from the boundary codes (bot, top), each -1 (odd), 0 (one-sided) or 1 (even).  Scheme fd02:
the second-order staggered operators (staggOps.F90) with PadeDerOps' per-code choices.
Scheme fourierColl (periodic, nz a power of two): Fourier collocation along z, each mode
multiplied by its factor (i k, -k^2, and the half-cell shifts e^{+-i k dz/2}).  Arrays are
Fortran-ordered (x fastest): cell fields (n1, n2, nz), edge fields (n1, n2, nz + 1), real
float64 or complex128, as CUDA torch tensors (asynchronous on the current stream) or host
numpy arrays (staged by the library).  The x-y extents are taken from the arrays.
"""
import ctypes

import numpy as np

from . import _lib as L
from ._base import buffer

fd02, cd06, fourierColl = 0, 1, 2


class Pade6stagg:
    """init / destroy / getModifiedWavenumbers / getApproxPoincareConstant and the generic
    ddz_C2E, ddz_E2C, interpz_C2E, interpz_E2C, d2dz2_C2C, d2dz2_E2E (REAL and CMPLX)."""

    def __init__(self):
        self._h = ctypes.c_void_p(None)
        self.isPeriodic = False

    def init(self, nz, dz, scheme=cd06, isPeriodic=False):
        """PadeDerOps.F90:57-124 with nz = gpC%zsz(3); returns 0 or the reference's code."""
        self.destroy()
        h = ctypes.c_void_p(None)
        rc = L.lib().pade_pade6stagg_init(ctypes.byref(h), int(nz), float(dz), int(scheme), int(bool(isPeriodic)))
        if rc == L.PADE_OK:
            self._h = h
            self.nz, self.dz, self.scheme, self.isPeriodic = nz, dz, scheme, bool(isPeriodic)
        return rc

    @property
    def handle(self):
        if not self._h.value:
            raise L.PadeError(L.PADE_EINVAL, "Pade6stagg used before init")
        return self._h

    def destroy(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pade_pade6stagg_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def _xy(self, a):
        shape = tuple(a.shape)
        if not isinstance(a, np.ndarray):  # torch tensors hold the Fortran array with reversed dims
            shape = tuple(reversed(shape))
        return shape[0], shape[1]

    def _apply(self, op, inp, out, bot, top):
        pi, ci, si, _ = buffer(inp, "input", True)
        po, co, so, _ = buffer(out, "output", True)
        if ci != co:
            raise TypeError("input and output must both be real or both complex")
        n1, n2 = self._xy(inp)
        stream = si if si is not None else so
        L.check(L.lib().pade_pade6stagg_apply(self.handle, op, int(ci), pi, po, n1, n2, int(bot), int(top), stream),
                f"Pade6stagg.{L.PADE6_OPS[op]}")

    def ddz_C2E(self, input, output, bot, top):
        self._apply(0, input, output, bot, top)

    def ddz_E2C(self, input, output, bot, top):
        self._apply(1, input, output, bot, top)

    def interpz_C2E(self, input, output, bot, top):
        self._apply(2, input, output, bot, top)

    def interpz_E2C(self, input, output, bot, top):
        self._apply(3, input, output, bot, top)

    def d2dz2_C2C(self, input, output, bot, top):
        self._apply(4, input, output, bot, top)

    def d2dz2_E2E(self, input, output, bot, top):
        self._apply(5, input, output, bot, top)

    def getModifiedWavenumbers(self, k):
        """PadeDerOps.F90:997-1016 (host)."""
        k = np.ascontiguousarray(k, dtype=np.float64)
        kp = np.empty_like(k)
        dp = ctypes.POINTER(ctypes.c_double)
        L.check(L.lib().pade_pade6stagg_getModifiedWavenumbers(self.handle, k.ctypes.data_as(dp),
                                                                kp.ctypes.data_as(dp), k.size),
                "Pade6stagg.getModifiedWavenumbers")
        return kp

    def getApproxPoincareConstant(self):
        """PadeDerOps.F90:1018-1032."""
        c = ctypes.c_double()
        L.check(L.lib().pade_pade6stagg_getApproxPoincareConstant(self.handle, ctypes.byref(c)),
                "Pade6stagg.getApproxPoincareConstant")
        return c.value
