"""Mirror of module FiltersMod (src/filters/filters.F90): type filters.

Per-direction filter selection: 1 "cf90", 2 "gaussian" (filters.F90:82-184); "lstsq" is
outside this library's scope.
"""
from . import _lib as L
from .cf90stuff import cf90
from .gaussianstuff import gaussian

METHODS = {"cf90": 1, "gaussian": 2, "lstsq": 3}


class filters:
    def init(self, nx, ny, nz, periodic_x, periodic_y, periodic_z, method_x, method_y, method_z):
        """init_serial (filters.F90:296-322)."""
        self.xsz = (nx, ny, nz)
        self.methods, self.ops = [], []
        codes = []
        for m in (method_x, method_y, method_z):  # every method is checked before any object is made
            code = METHODS.get(m.strip().lower())
            if code is None or code == 3:
                raise L.PadeError(L.PADE_ENOTSUP if code == 3 else L.PADE_EINVAL, f"filters.init: method {m!r}")
            codes.append(code)
        for n, per, code in ((nx, periodic_x, codes[0]), (ny, periodic_y, codes[1]), (nz, periodic_z, codes[2])):
            o = cf90() if code == 1 else gaussian()
            ierr = o.init(n, per)
            if ierr != 0:
                raise L.PadeError(ierr, "filters.init")
            self.methods.append(code)
            self.ops.append(o)

    def getMethodx(self):
        return self.methods[0]

    def getMethody(self):
        return self.methods[1]

    def getMethodz(self):
        return self.methods[2]

    def _f(self, d, f, ff, bc1, bcn):
        na, nb = [s for k, s in enumerate(self.xsz) if k != d - 1]
        getattr(self.ops[d - 1], f"filter{d}")(f, ff, na, nb, bc1, bcn)

    def filterx(self, f, ff, bc1=None, bcn=None):
        self._f(1, f, ff, bc1, bcn)

    def filtery(self, f, ff, bc1=None, bcn=None):
        self._f(2, f, ff, bc1, bcn)

    def filterz(self, f, ff, bc1=None, bcn=None):
        self._f(3, f, ff, bc1, bcn)

    def destroy(self):
        for o in self.ops:
            o.destroy()
        self.ops = []
