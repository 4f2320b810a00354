"""Mirror of module spectralMod (src/incompressible/spectral.F90): type spectral.

The x-y Fourier layer of the incompressible solver for grids periodic in x and y:
``fft`` = r2c along x then forward c2c along y, ``ifft`` = backward c2c along y, optional
oddball zeroing, c2r along x, times 1/(nx ny) (fft_3d.F90:616-663).  Arrays are CUDA
torch tensors in Fortran order (x fastest): physical (nx, ny, nz) float64, spectral
(nx/2+1, ny, nz) complex128.  Transform lengths must be powers of two.
"""
import ctypes

import numpy as np

from . import _lib as L
from ._base import buffer


def GetWaveNums(n, dx):
    """spectral.F90:1748-1764 (host)."""
    k = np.empty(n)
    L.check(L.lib().pade_wavenumbers(int(n), float(dx), k.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
            "GetWaveNums")
    return k


def getmodCD06stagg(k, dz):
    """PadeDerOps.F90:1034-1053 (host)."""
    k = np.ascontiguousarray(k, dtype=np.float64)
    kp = np.empty_like(k)
    dp = ctypes.POINTER(ctypes.c_double)
    L.check(L.lib().pade_modified_wavenumbers_cd06stagg(k.ctypes.data_as(dp), k.size, float(dz), kp.ctypes.data_as(dp)),
            "getmodCD06stagg")
    return kp


def _dev(a, what):
    p, cplx, stream, _ = buffer(a, what, complex_ok=True)
    if stream is None:
        raise TypeError(f"{what} must be a CUDA tensor")
    return p, cplx, stream


class spectral:
    """Two-periodic spectral type: init, fft, ifft, k1/k2 wavenumbers."""

    def __init__(self):
        self._h = ctypes.c_void_p(None)

    def init(self, nx, ny, nz, dx, dy, fixOddball=True):
        """spectral.F90:867-1215 for the x-y periodic (two-dimensional transform) case."""
        self.destroy()
        h = ctypes.c_void_p(None)
        L.check(L.lib().pade_spectral_init(ctypes.byref(h), int(nx), int(ny), int(nz), float(dx), float(dy),
                                           int(bool(fixOddball))), "spectral.init")
        self._h = h
        self.nx_g, self.ny_g, self.nz_g = nx, ny, nz
        self.physical_shape = (nx, ny, nz)
        self.spectral_shape = (nx // 2 + 1, ny, nz)
        k1 = np.empty(nx // 2 + 1)
        k2 = np.empty(ny)
        dp = ctypes.POINTER(ctypes.c_double)
        L.check(L.lib().pade_spectral_get_wavenumbers(h, k1.ctypes.data_as(dp), k2.ctypes.data_as(dp)))
        self.k1_1d, self.k2_1d = k1, k2

    @property
    def handle(self):
        if not self._h.value:
            raise L.PadeError(L.PADE_EINVAL, "spectral used before init")
        return self._h

    def fft(self, arr_in, arr_out):
        pi, _, s = _dev(arr_in, "arr_in")
        po, _, _ = _dev(arr_out, "arr_out")
        L.check(L.lib().pade_spectral_fft(self.handle, pi, po, s), "spectral.fft")

    def ifft(self, arr_in, arr_out, setOddball=False):
        pi, _, s = _dev(arr_in, "arr_in")
        po, _, _ = _dev(arr_out, "arr_out")
        L.check(L.lib().pade_spectral_ifft(self.handle, pi, po, int(bool(setOddball)), s), "spectral.ifft")

    # ---- the fused spectral layer (pointwise multipliers folded into the transforms) ----
    def ifft_ik(self, arr_in, arr_out, d):
        """ifft(mTimes_ik1_oop(arr_in)) for d = 1, ifft(mTimes_ik2_oop(arr_in)) for d = 2."""
        pi, _, s = _dev(arr_in, "arr_in")
        po, _, _ = _dev(arr_out, "arr_out")
        L.check(L.lib().pade_spectral_ifft_ik(self.handle, pi, po, int(d), s), "spectral.ifft_ik")

    def ifft_and_ddx(self, arr_in, arr_out, arr_out_dx):
        """ifft(arr_in) and ifft(mTimes_ik1_oop(arr_in))."""
        pi, _, s = _dev(arr_in, "arr_in")
        po, _, _ = _dev(arr_out, "arr_out")
        pd, _, _ = _dev(arr_out_dx, "arr_out_dx")
        L.check(L.lib().pade_spectral_ifft_and_ddx(self.handle, pi, po, pd, s), "spectral.ifft_and_ddx")

    def fft_two(self, in1, in2, out1, out2):
        """fft(in1) -> out1 and fft(in2) -> out2."""
        p1, _, s = _dev(in1, "in1")
        p2, _, _ = _dev(in2, "in2")
        q1, _, _ = _dev(out1, "out1")
        q2, _, _ = _dev(out2, "out2")
        L.check(L.lib().pade_spectral_fft_two(self.handle, p1, p2, q1, q2, s), "spectral.fft_two")

    def ifft_two(self, in1, d1, in2, d2, out1, out2):
        """ifft of (i k_d1) in1 and (i k_d2) in2 (d = 0: no multiplier)."""
        p1, _, s = _dev(in1, "in1")
        p2, _, _ = _dev(in2, "in2")
        q1, _, _ = _dev(out1, "out1")
        q2, _, _ = _dev(out2, "out2")
        L.check(L.lib().pade_spectral_ifft_two(self.handle, p1, int(d1), p2, int(d2), q1, q2, s), "spectral.ifft_two")

    def ifft_testfilter(self, arr_in, arr_out, filtfact=2.0):
        """ifft(TestFilter_oop(arr_in)) with the cutoff of InitTestFilter(filtfact)."""
        pi, _, s = _dev(arr_in, "arr_in")
        po, _, _ = _dev(arr_out, "arr_out")
        L.check(L.lib().pade_spectral_ifft_testfilter(self.handle, pi, po, float(filtfact), s),
                "spectral.ifft_testfilter")

    def destroy(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pade_spectral_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
