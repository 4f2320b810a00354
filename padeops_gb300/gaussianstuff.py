"""Mirror of module gaussianstuff (src/filters/gaussian.F90): type gaussian."""
from . import _lib as L
from ._base import PadeObject


class gaussian(PadeObject):
    """Explicit 9-point Gaussian filter of width 4 dx (gaussian.F90:16-43)."""

    def init(self, n, periodic):
        """gaussian.F90:74-93; returns ierr (0)."""
        self.n = n
        return self._init(L.lib().pade_gaussian_init, int(n), int(bool(periodic)))

    def _f(self, name, f, ff, na, nb, bc1_, bcn_, cplx=False):
        Lb = L.lib()
        fn = getattr(Lb, f"pade_gaussian_{name}")
        cfn = getattr(Lb, f"pade_gaussian_{name}_cmplx") if cplx else None
        self._call(fn, name, f, ff, na, nb, 0 if bc1_ is None else int(bc1_), 0 if bcn_ is None else int(bcn_),
                   complex_fn=cfn)

    def filter1(self, f, ff, na, nb, bc1_=None, bcn_=None):
        self._f("filter1", f, ff, na, nb, bc1_, bcn_)

    def filter2(self, f, ff, na, nb, bc1_=None, bcn_=None):
        self._f("filter2", f, ff, na, nb, bc1_, bcn_)

    def filter3(self, f, ff, na, nb, bc1_=None, bcn_=None):
        self._f("filter3", f, ff, na, nb, bc1_, bcn_, cplx=True)
