"""Mirror of module cd06staggstuff (src/derivatives/cd06stagg.F90): type cd06stagg."""
from . import _lib as L
from ._base import PadeObject


class cd06stagg(PadeObject):
    """Staggered 6th-order compact operators between cells (n points) and edges (n+1).

    init(n, dx) is the periodic constructor; init(n, dx, isTopEven, isBotEven[,
    isTopSided, isBotSided]) the non-periodic one (the reference's generic init).
    Every operator accepts REAL or COMPLEX arrays (the reference's generic overloads).
    """

    def init(self, nx, dx, isTopEven=None, isBotEven=None, isTopSided=False, isBotSided=False):
        self.n = nx
        if isTopEven is None and isBotEven is None:
            self.periodic = True
            return self._init(L.lib().pade_cd06stagg_init_periodic, int(nx), float(dx))
        self.periodic = False
        return self._init(L.lib().pade_cd06stagg_init_nonperiodic, int(nx), float(dx), int(bool(isTopEven)),
                          int(bool(isBotEven)), int(bool(isTopSided)), int(bool(isBotSided)))

    def _op(self, name, fi, fo, n1, n2):
        Lb = L.lib()
        self._call(getattr(Lb, f"pade_cd06stagg_{name}"), name, fi, fo, n1, n2,
                   complex_fn=getattr(Lb, f"pade_cd06stagg_{name}_cmplx"))

    def ddz_E2C(self, fE, dfC, n1, n2):
        self._op("ddz_E2C", fE, dfC, n1, n2)

    def ddz_C2E(self, fC, dfE, n1, n2):
        self._op("ddz_C2E", fC, dfE, n1, n2)

    def ddz_C2C(self, fC, dfC, n1, n2):
        self._op("ddz_C2C", fC, dfC, n1, n2)

    def ddz_E2E(self, fE, dfE, n1, n2):
        self._op("ddz_E2E", fE, dfE, n1, n2)

    def d2dz2_C2C(self, fC, d2fC, n1, n2):
        self._op("d2dz2_C2C", fC, d2fC, n1, n2)

    def d2dz2_E2E(self, fE, d2fE, n1, n2):
        self._op("d2dz2_E2E", fE, d2fE, n1, n2)

    def InterpZ_E2C(self, fE, IfC, n1, n2):
        self._op("InterpZ_E2C", fE, IfC, n1, n2)

    def InterpZ_C2E(self, fC, IfE, n1, n2):
        self._op("InterpZ_C2E", fC, IfE, n1, n2)
