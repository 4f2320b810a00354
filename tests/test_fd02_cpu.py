"""Pade6stagg's second-order scheme (fd02) on the host (no GPU): the library's operator
definitions (pade_plan_check, family 5) against the numpy restatement of staggOps.F90 and
PadeDerOps.F90 (oracle/fd02_oracle.py), and the restatement's known answers."""
import numpy as np
import pytest

from oracle import fd02_oracle as FO
from padeops_gb300 import _lib as L
from tests.libhost import params, plan_apply_lines

# Pade6stagg operation -> the library's staggered opcode (pade_apply numbering)
OPCODE = {0: 1, 1: 0, 2: 7, 3: 6, 4: 4, 5: 5}
E_IN = {0: False, 1: True, 2: False, 3: True, 4: False, 5: True}


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("op", range(6))
def test_operator_definitions_match_the_restatement(op, periodic):
    nz, dz = 12, 0.37
    rng = np.random.default_rng(op + 10 * periodic)
    lines = rng.standard_normal((5, nz + (1 if E_IN[op] else 0)))
    prm = params("fd02", nz, dz, periodic)
    codes = [(0, 0)] if periodic else [(b, t) for b in (-1, 0, 1) for t in (-1, 0, 1)] + [(2, 0), (1, 7)]
    for bot, top in codes:
        ref = FO.apply(op, lines, dz, periodic, bot, top)
        got = plan_apply_lines("fd02", prm, OPCODE[op], bot, top, lines)
        assert got.shape == ref.shape
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(got - ref).max() <= 1e-14 * scale, (bot, top)


def test_known_answers():
    nz, dz = 10, 0.25
    zc = (np.arange(nz) + 0.5) * dz  # cells
    ze = np.arange(nz + 1) * dz      # edges
    a, b, c = 0.7, -1.3, 0.4
    lin_e, lin_c = a + b * ze, a + b * zc
    assert np.allclose(FO.ddz_E2C(lin_e, dz), b, rtol=0, atol=1e-14)
    assert np.allclose(FO.interpz_E2C(lin_e), lin_c, rtol=0, atol=1e-14)
    # interior of C2E derivative / interpolation of a linear profile
    assert np.allclose(FO.ddz_C2E(lin_c, dz, bot=-1, top=-1)[1:-1], b, rtol=0, atol=1e-13)
    assert np.allclose(FO.interpz_C2E(lin_c, bot=0, top=0), lin_e, rtol=0, atol=1e-14)  # one-sided ends are exact
    quad_c = c * zc ** 2
    assert np.allclose(FO.d2dz2_C2C(quad_c, dz, bot=1, top=1)[1:-1], 2 * c, rtol=0, atol=1e-12)
    # evenness rules at the walls: an odd field's edge value 0, an even field's edge derivative 0
    f = np.cos(np.pi * zc / (nz * dz))
    e = FO.ddz_C2E(f, dz, bot=1, top=1)
    assert e[0] == 0.0 and e[-1] == 0.0
    assert FO.interpz_C2E(f, bot=-1, top=-1)[0] == 0.0


def test_family_exposed():
    assert L.FAMILY["fd02"] == 5
