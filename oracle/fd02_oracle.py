"""numpy restatement of Pade6stagg's second-order staggered scheme (fd02).

TEST INFRASTRUCTURE ONLY: the tests use it as the checker; the library never calls it.

The operators are staggOps' (src/incompressible/staggOps.F90), selected and post-processed
per boundary-code pair (bot, top) as the fd02 branches of src/incompressible/PadeDerOps.F90
do.  Arrays are Fortran-shaped (n1, n2, nz) cells / (n1, n2, nz + 1) edges, real or complex;
every operator acts along the last axis.  Combinations the reference has no operator for
return zeros (PadeDerOps sets output = 0, or leaves it unassigned).

Parity pinning: the formulas are copied as data from the reference files cited per
function; the operators are explicit stencils, so their known answers (exact derivatives of
linear / quadratic profiles in the interior, the evenness rules at the ends) are checked in
tests/test_fd02_cpu.py.
"""
import numpy as np

VALID = (-1, 0, 1)


def ddz_E2C(fE, dz, periodic=False, bot=1, top=1):
    """staggOps.F90:54-64; every (bot, top) uses it (PadeDerOps.F90:583-585)."""
    return (fE[..., 1:] - fE[..., :-1]) * (1.0 / dz)


def interpz_E2C(fE, periodic=False, bot=1, top=1):
    """staggOps.F90:390-399 (PadeDerOps.F90:888-897)."""
    return 0.5 * (fE[..., :-1] + fE[..., 1:])


def _c2e_flags(bot, top):
    """(isTopEven, isBotEven) of the fd02 ddz_C2E calls, PadeDerOps.F90:419-445."""
    table = {(-1, -1): (False, False), (-1, 0): (True, False), (-1, 1): (True, False),
             (0, -1): (False, True), (0, 0): (False, True), (0, 1): (True, True),
             (1, -1): (False, True), (1, 0): (False, True), (1, 1): (True, True)}
    return table[(bot, top)]


def ddz_C2E(fC, dz, periodic=False, bot=1, top=1):
    """staggOps.F90:78-107."""
    nz = fC.shape[-1]
    out = np.zeros(fC.shape[:-1] + (nz + 1,), dtype=fC.dtype)
    if not periodic and (bot not in VALID or top not in VALID):
        return out
    out[..., 1:nz] = fC[..., 1:] - fC[..., :-1]
    if periodic:
        out[..., 0] = fC[..., 0] - fC[..., nz - 1]
        out[..., nz] = out[..., 0]
    else:
        top_even, bot_even = _c2e_flags(bot, top)
        out[..., 0] = 0.0 if bot_even else 2.0 * fC[..., 0]
        out[..., nz] = 0.0 if top_even else -2.0 * fC[..., nz - 1]
    return out * (1.0 / dz)


def interpz_C2E(fC, periodic=False, bot=1, top=1):
    """staggOps.F90:431-448 (BotVal = TopVal = 0) and the overrides of PadeDerOps.F90:703-738."""
    nz = fC.shape[-1]
    out = np.zeros(fC.shape[:-1] + (nz + 1,), dtype=fC.dtype)
    if not periodic and (bot not in VALID or top not in VALID):
        return out
    out[..., 1:nz] = 0.5 * (fC[..., :-1] + fC[..., 1:])
    if periodic:
        out[..., 0] = 0.5 * (fC[..., 0] + fC[..., nz - 1])
        out[..., nz] = out[..., 0]
        return out
    if top == 0:
        out[..., nz] = 2.0 * fC[..., nz - 1] - out[..., nz - 1]
    elif top == 1:
        out[..., nz] = fC[..., nz - 1]
    if bot == 0:
        out[..., 0] = 2.0 * fC[..., 0] - out[..., 1]
    elif bot == 1:
        out[..., 0] = fC[..., 0]
    return out


def d2dz2_C2C(fC, dz, periodic=False, bot=1, top=1):
    """staggOps.F90:235-264 (isTopEven = top == 1, isBotEven = bot == 1: PadeDerOps.F90:159-183;
    a one-sided or invalid code gives zeros)."""
    nz = fC.shape[-1]
    out = np.zeros_like(fC)
    if not periodic and (bot not in (-1, 1) or top not in (-1, 1)):
        return out
    out[..., 1:nz - 1] = fC[..., 2:] - 2.0 * fC[..., 1:nz - 1] + fC[..., :nz - 2]
    if periodic:
        out[..., 0] = fC[..., 1] - 2.0 * fC[..., 0] + fC[..., nz - 1]
        out[..., nz - 1] = fC[..., 0] - 2.0 * fC[..., nz - 1] + fC[..., nz - 2]
    else:
        out[..., 0] = fC[..., 1] - fC[..., 0] if bot == 1 else fC[..., 1] - 3.0 * fC[..., 0]
        out[..., nz - 1] = fC[..., nz - 2] - fC[..., nz - 1] if top == 1 else fC[..., nz - 2] - 3.0 * fC[..., nz - 1]
    return out * (1.0 / (dz * dz))


def d2dz2_E2E(fE, dz, periodic=False, bot=1, top=1):
    """staggOps.F90:297-326 (evenness as in d2dz2_C2C: PadeDerOps.F90:283-312)."""
    nE = fE.shape[-1]
    out = np.zeros_like(fE)
    if not periodic and (bot not in (-1, 1) or top not in (-1, 1)):
        return out
    out[..., 1:nE - 1] = fE[..., 2:] - 2.0 * fE[..., 1:nE - 1] + fE[..., :nE - 2]
    if periodic:
        out[..., 0] = fE[..., 1] - 2.0 * fE[..., 0] + fE[..., nE - 2]
        out[..., nE - 1] = fE[..., 1] - 2.0 * fE[..., nE - 1] + fE[..., nE - 2]
    else:
        out[..., 0] = 2.0 * (fE[..., 1] - fE[..., 0]) if bot == 1 else 0.0
        out[..., nE - 1] = 2.0 * (fE[..., nE - 2] - fE[..., nE - 1]) if top == 1 else 0.0
    return out * (1.0 / (dz * dz))


# Pade6stagg operation index (pade_pade6stagg_apply) -> (oracle function, takes dz, input on edges)
OPS = {0: (ddz_C2E, True, False), 1: (ddz_E2C, True, True), 2: (interpz_C2E, False, False),
       3: (interpz_E2C, False, True), 4: (d2dz2_C2C, True, False), 5: (d2dz2_E2E, True, True)}


def apply(op, f, dz, periodic, bot, top):
    fn, has_dz, _ = OPS[op]
    return fn(f, dz, periodic, bot, top) if has_dz else fn(f, periodic, bot, top)
