"""Mirror of module PadePoissonMod (src/incompressible/PadePoisson.F90): type padepoisson.

Periodic in z (``PeriodicInZ = .true.``) or with walls at z = 0 and Lz (``PeriodicInZ =
.false.``, with the optional Stokes-pressure wall correction): the pressure projection
that is consistent with the staggered CD06 z derivative, and the divergence check.  uhat
and vhat are complex (nx/2+1, ny, nz) CUDA tensors, what is complex (nx/2+1, ny, nz+1);
all are updated in place; getPressure / getPressureAndUpdateRHS return the pressure in
physical space.
"""
import ctypes

import numpy as np

from . import _lib as L
from .spectralMod import _dev


class padepoisson:
    def __init__(self):
        self._h = ctypes.c_void_p(None)

    def init(self, dx, dy, dz, sp, PeriodicInZ=True, computeStokesPressure=False, Lz=None):
        """PadePoisson.F90:130-318 (+ InitPeriodicPoissonSolver 76-128 when PeriodicInZ)."""
        self.destroy()
        h = ctypes.c_void_p(None)
        if PeriodicInZ:
            L.check(L.lib().pade_poisson_periodic_init(ctypes.byref(h), sp.handle, float(dx), float(dy), float(dz)),
                    "padepoisson.init")
        else:
            lz = float(Lz) if Lz is not None else float(dz) * sp.nz_g
            L.check(L.lib().pade_poisson_wall_init(ctypes.byref(h), sp.handle, float(dx), float(dy), float(dz), lz,
                                                   int(bool(computeStokesPressure))), "padepoisson.init")
        self._h = h
        self._sp = sp  # the handle keeps a pointer to it
        self.PeriodicInZ = bool(PeriodicInZ)
        self.k3mod = None
        if PeriodicInZ:
            k3 = np.empty(sp.nz_g)
            L.check(L.lib().pade_poisson_get_modified_k3(h, k3.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
            self.k3mod = k3

    @property
    def handle(self):
        if not self._h.value:
            raise L.PadeError(L.PADE_EINVAL, "padepoisson used before init")
        return self._h

    def PressureProjection(self, uhat, vhat, what):
        pu, _, s = _dev(uhat, "uhat")
        pv, _, _ = _dev(vhat, "vhat")
        pw, _, _ = _dev(what, "what")
        L.check(L.lib().pade_poisson_projection(self.handle, pu, pv, pw, s), "PressureProjection")

    def getPressure(self, uhat, vhat, what, pressure):
        """PadePoisson.F90:716-898: pressure (real (nx, ny, nz) CUDA tensor, physical space)
        of the right-hand sides uhat, vhat, what, which are left unchanged."""
        pu, _, s = _dev(uhat, "uhat")
        pv, _, _ = _dev(vhat, "vhat")
        pw, _, _ = _dev(what, "what")
        pp, _, _ = _dev(pressure, "pressure")
        L.check(L.lib().pade_poisson_get_pressure(self.handle, pu, pv, pw, pp, s), "getPressure")

    def getPressureAndUpdateRHS(self, uhat, vhat, what, pressure):
        """PadePoisson.F90:900-1163: the pressure, and uhat, vhat, what projected in place."""
        pu, _, s = _dev(uhat, "uhat")
        pv, _, _ = _dev(vhat, "vhat")
        pw, _, _ = _dev(what, "what")
        pp, _, _ = _dev(pressure, "pressure")
        L.check(L.lib().pade_poisson_get_pressure_and_update_rhs(self.handle, pu, pv, pw, pp, s),
                "getPressureAndUpdateRHS")

    def DivergenceCheck(self, uhat, vhat, what, divergence, fixDiv=False):
        """Fills divergence; returns max(divergence) (the reference keeps it internal)."""
        pu, _, s = _dev(uhat, "uhat")
        pv, _, _ = _dev(vhat, "vhat")
        pw, _, _ = _dev(what, "what")
        pd, _, _ = _dev(divergence, "divergence")
        m = ctypes.c_double(0.0)
        L.check(L.lib().pade_poisson_divergence_check(self.handle, pu, pv, pw, pd, int(bool(fixDiv)),
                                                       ctypes.byref(m), s), "DivergenceCheck")
        return m.value

    def destroy(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pade_poisson_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
