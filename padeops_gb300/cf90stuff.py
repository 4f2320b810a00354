"""Mirror of module cf90stuff (src/filters/cf90.F90): type cf90."""
from . import _lib as L
from ._base import PadeObject


class cf90(PadeObject):
    """8th-order compact filter with 90 % truncation (alpha = 0.66624, beta = 0.16688)."""

    def init(self, n, periodic):
        """cf90.F90:107-175; returns ierr (0 or 7)."""
        self.n = n
        return self._init(L.lib().pade_cf90_init, int(n), int(bool(periodic)))

    def _f(self, name, f, ff, na, nb, bc1_, bcn_, cplx=False):
        Lb = L.lib()
        fn = getattr(Lb, f"pade_cf90_{name}")
        cfn = getattr(Lb, f"pade_cf90_{name}_cmplx") if cplx else None
        self._call(fn, name, f, ff, na, nb, 0 if bc1_ is None else int(bc1_), 0 if bcn_ is None else int(bcn_),
                   complex_fn=cfn)

    def filter1(self, f, ff, na, nb, bc1_=None, bcn_=None):
        self._f("filter1", f, ff, na, nb, bc1_, bcn_)

    def filter2(self, f, ff, na, nb, bc1_=None, bcn_=None):
        self._f("filter2", f, ff, na, nb, bc1_, bcn_)

    def filter3(self, f, ff, na, nb, bc1_=None, bcn_=None):
        """Generic over REAL and CMPLX arrays like the reference (cf90.F90:99)."""
        self._f("filter3", f, ff, na, nb, bc1_, bcn_, cplx=True)
