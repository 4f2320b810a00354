"""GB300-native compact operators of PadeOps behind the reference's module API.

Modules mirror the reference Fortran modules: ``cd06stuff.cd06``, ``cd10stuff.cd10``,
``cf90stuff.cf90``, ``gaussianstuff.gaussian``, ``cd06staggstuff.cd06stagg``, igrid's z-operator
facade ``PadeDerOps.Pade6stagg``, the
dispatchers ``DerivativesMod.derivatives`` / ``FiltersMod.filters``, the spectral layer
``spectralMod.spectral``, ``PadePoissonMod.padepoisson``, ``PoissonPeriodicMod.PoissonPeriodic``
the one-rank pencil transposes in ``decomp_2d`` and the periodic LES step
``IncompressibleGrid.igrid``.  The
compute path is ``libpadeops_gb300.so`` (hand-written sm_103a kernels behind a C ABI).
"""
from ._lib import PATH_DF, PATH_FP32, PATH_NATIVE, PadeError  # noqa: F401
from .cd06staggstuff import cd06stagg  # noqa: F401
from .DerivativesMod import derivatives  # noqa: F401
from .FiltersMod import filters  # noqa: F401
from .cd06stuff import cd06  # noqa: F401
from .cd10stuff import cd10  # noqa: F401
from .cf90stuff import cf90  # noqa: F401
from .gaussianstuff import gaussian  # noqa: F401
from .IncompressibleGrid import igrid  # noqa: F401
from .PadeDerOps import Pade6stagg  # noqa: F401
from .PadePoissonMod import padepoisson  # noqa: F401
from .PoissonPeriodicMod import PoissonPeriodic  # noqa: F401
from .spectralMod import spectral  # noqa: F401

__all__ = ["cd06", "cd10", "cf90", "gaussian", "cd06stagg", "Pade6stagg", "derivatives", "filters", "spectral",
           "padepoisson", "PoissonPeriodic", "igrid", "PadeError", "PATH_DF", "PATH_NATIVE", "PATH_FP32"]
