"""Mirror of module cd06stuff (src/derivatives/cd06.F90): type cd06."""
from . import _lib as L
from ._base import PadeObject


class cd06(PadeObject):
    """6th-order collocated compact first derivative (Lele 1992).

    Periodic lines use the cyclic tridiagonal system (alpha = 1/3), non-periodic lines the
    one-sided w1..w3 closures (cd06.F90:14-59).  d2d1..d2d3 complete the reference's
    periodic second derivative (incomplete upstream, cd06.F90:745-773).
    """

    def init(self, n, dx, periodic, bc1=0, bcn=0):
        """cd06.F90:129-201; returns ierr (0, 2 or 3) like the reference."""
        self.n = n
        return self._init(L.lib().pade_cd06_init, int(n), float(dx), int(bool(periodic)), int(bc1), int(bcn))

    def GetSize(self):
        return self.n

    def dd1(self, f, df, na, nb):
        self._call(L.lib().pade_cd06_dd1, "dd1", f, df, na, nb)

    def dd2(self, f, df, na, nb):
        self._call(L.lib().pade_cd06_dd2, "dd2", f, df, na, nb)

    def dd3(self, f, df, na, nb):
        self._call(L.lib().pade_cd06_dd3, "dd3", f, df, na, nb)

    def d2d1(self, f, df, na, nb):
        self._call(L.lib().pade_cd06_d2d1, "d2d1", f, df, na, nb)

    def d2d2(self, f, df, na, nb):
        self._call(L.lib().pade_cd06_d2d2, "d2d2", f, df, na, nb)

    def d2d3(self, f, df, na, nb):
        self._call(L.lib().pade_cd06_d2d3, "d2d3", f, df, na, nb)
