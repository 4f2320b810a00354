"""Mirror of module cd10stuff (src/derivatives/cd10.F90): type cd10."""
from . import _lib as L
from ._base import PadeObject


class cd10(PadeObject):
    """10th-order collocated compact first and second derivatives (Lele 1992).

    Periodic: cyclic pentadiagonal; non-periodic: the nine (bc1, bcn) factorisations with
    bc in {0 one-sided, 1 symmetric, -1 antisymmetric} (cd10.F90:195-315).
    """

    def init(self, n, dx, periodic, bc1=0, bcn=0):
        """cd10.F90:195-315; returns ierr (0 or 2)."""
        self.n = n
        return self._init(L.lib().pade_cd10_init, int(n), float(dx), int(bool(periodic)), int(bc1), int(bcn))

    def GetSize(self):
        return self.n

    def _d(self, name, f, df, na, nb, bc1_, bcn_):
        fn = getattr(L.lib(), f"pade_cd10_{name}")
        self._call(fn, name, f, df, na, nb, 0 if bc1_ is None else int(bc1_), 0 if bcn_ is None else int(bcn_))

    def dd1(self, f, df, na, nb, bc1_=None, bcn_=None):
        self._d("dd1", f, df, na, nb, bc1_, bcn_)

    def dd2(self, f, df, na, nb, bc1_=None, bcn_=None):
        self._d("dd2", f, df, na, nb, bc1_, bcn_)

    def dd3(self, f, df, na, nb, bc1_=None, bcn_=None):
        self._d("dd3", f, df, na, nb, bc1_, bcn_)

    def d2d1(self, f, df, na, nb, bc1_=None, bcn_=None):
        self._d("d2d1", f, df, na, nb, bc1_, bcn_)

    def d2d2(self, f, df, na, nb, bc1_=None, bcn_=None):
        self._d("d2d2", f, df, na, nb, bc1_, bcn_)

    def d2d3(self, f, df, na, nb, bc1_=None, bcn_=None):
        self._d("d2d3", f, df, na, nb, bc1_, bcn_)
