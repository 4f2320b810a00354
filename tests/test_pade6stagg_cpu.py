"""Pade6stagg host-side behaviour (no GPU): the second-order scheme's modified
wavenumbers (getmodFD02stagg, PadeDerOps.F90:1055-1074), the Poincare constants of each
scheme (PadeDerOps.F90:1018-1032) and the reference's init error codes (434, 323)."""
import numpy as np
import pytest

import padeops_gb300 as P
from padeops_gb300 import _lib as L


def test_fd02_modified_wavenumbers_and_constants():
    p = P.Pade6stagg()
    dz = 0.1
    assert p.init(40, dz, P.PadeDerOps.fd02, True) == 0
    k = np.linspace(0, np.pi / dz, 17)
    assert np.allclose(p.getModifiedWavenumbers(k), 2 * np.sin(k * dz / 2) / dz, rtol=1e-15, atol=0)
    assert p.getApproxPoincareConstant() == 1.0 / np.sqrt(3.0)
    assert P.Pade6stagg().init(2, dz, P.PadeDerOps.fd02, False) == L.PADE_EINVAL  # fd02 needs nz >= 3


def test_init_error_codes():
    assert P.Pade6stagg().init(16, 0.1, 7, True) == 434
    assert P.Pade6stagg().init(16, 0.1, 7, False) == 323
    assert P.Pade6stagg().init(16, 0.1, P.PadeDerOps.fourierColl, False) == 323
    assert P.Pade6stagg().init(16, 0.1, P.PadeDerOps.fourierColl, True) == 0
    assert P.Pade6stagg().init(24, 0.1, P.PadeDerOps.fourierColl, True) == L.PADE_ENOTSUP  # FFT lengths: 2^k
    assert P.Pade6stagg().init(16, -1.0, P.PadeDerOps.cd06, True) == L.PADE_EINVAL
