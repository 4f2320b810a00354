"""Mirror of module DerivativesMod (src/derivatives/derivatives.F90): type derivatives.

Per-direction method selection over the compact objects: method 1 "cd10", 2 "cd06"
(derivatives.F90:14-56).  "four" (Fourier collocation) and "cheb" are outside this
library's scope and raise like the reference's GracefulExit for unsupported methods.
Sizes follow the serial constructor: x/y/z pencils all span the full grid on one GPU.
"""
from . import _lib as L
from .cd06stuff import cd06
from .cd10stuff import cd10

METHODS = {"cd10": 1, "cd06": 2, "four": 3, "cheb": 4}


class derivatives:
    def __init__(self):
        self.initialized = False

    def init(self, nx, ny, nz, dx, dy, dz, periodic_x, periodic_y, periodic_z, method_x, method_y, method_z):
        """init_serial (derivatives.F90:140-187)."""
        self.xsz = self.ysz = self.zsz = (nx, ny, nz)
        self.methods = []
        self.ops = []
        codes = []
        for m in (method_x, method_y, method_z):  # every method is checked before any object is made
            code = METHODS.get(m.strip().lower())
            if code is None:
                raise L.PadeError(L.PADE_EINVAL, f"derivatives.init: unknown method {m!r}")
            if code in (3, 4):
                raise L.PadeError(L.PADE_ENOTSUP, f"derivatives.init: method {m!r} is not provided on this path")
            codes.append(code)
        for n, h, per, code in ((nx, dx, periodic_x, codes[0]), (ny, dy, periodic_y, codes[1]),
                                (nz, dz, periodic_z, codes[2])):
            o = cd10() if code == 1 else cd06()
            ierr = o.init(n, h, per)
            if ierr != 0:
                raise L.PadeError(ierr, "derivatives.init")
            self.methods.append(code)
            self.ops.append(o)
        self.initialized = True

    def getMethodx(self):
        return self.methods[0]

    def getMethody(self):
        return self.methods[1]

    def getMethodz(self):
        return self.methods[2]

    def _d1(self, d, f, df, bc1, bcn):
        o = self.ops[d - 1]
        na, nb = [s for k, s in enumerate(self.xsz) if k != d - 1]
        name = f"dd{d}"
        if self.methods[d - 1] == 1:
            if bc1 is not None and bcn is not None:
                getattr(o, name)(f, df, na, nb, bc1, bcn)
            else:
                getattr(o, name)(f, df, na, nb)
        else:
            getattr(o, name)(f, df, na, nb)

    def _d2(self, d, f, df, bc1, bcn):
        if self.methods[d - 1] == 2:
            # derivatives.F90:525 -- the reference refuses CD06 second derivatives
            raise L.PadeError(21, "CD06 is incomplete right now")
        o = self.ops[d - 1]
        na, nb = [s for k, s in enumerate(self.xsz) if k != d - 1]
        getattr(o, f"d2d{d}")(f, df, na, nb, bc1, bcn)

    def ddx(self, f, dfdx, bc1=None, bcn=None):
        self._d1(1, f, dfdx, bc1, bcn)

    def ddy(self, f, dfdy, bc1=None, bcn=None):
        self._d1(2, f, dfdy, bc1, bcn)

    def ddz(self, f, dfdz, bc1=None, bcn=None):
        self._d1(3, f, dfdz, bc1, bcn)

    def d2dx2(self, f, d2f, bc1=None, bcn=None):
        self._d2(1, f, d2f, bc1, bcn)

    def d2dy2(self, f, d2f, bc1=None, bcn=None):
        self._d2(2, f, d2f, bc1, bcn)

    def d2dz2(self, f, d2f, bc1=None, bcn=None):
        self._d2(3, f, d2f, bc1, bcn)

    def destroy(self):
        for o in getattr(self, "ops", []):
            o.destroy()
        self.ops = []
        self.initialized = False
