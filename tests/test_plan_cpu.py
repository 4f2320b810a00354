"""The library's operator plans (operator tables, banded LU, cyclic Woodbury terms),
evaluated on the CPU through the host-only pade_plan_check entry, against the oracle.

This validates every operator definition of the library without a GPU; the GPU parity
tests then only have to pin the kernels.
"""
import itertools

import numpy as np
import pytest

from tests.fields import relerr
from tests import libhost as H

BCS = [0, 1, -1]
TOL = 1e-13


def lines_for(nin, nlines=5, seed=0):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, nin)
    base = [np.sin(2 * np.pi * x * (k + 1) + k) for k in range(nlines - 1)]
    return np.stack(base + [rng.standard_normal(nin)])


def oracle_lines(fn, lines):
    # oracle works on Fortran arrays (n, nlines) along dir=1
    return np.stack([fn(l).ravel() for l in lines])


def tol_for(order, n):
    return TOL if order < 2 else max(TOL, 2e-13 * n * n / 64)


@pytest.mark.parametrize("n", [6, 7, 16, 64])
@pytest.mark.parametrize("order", [1, 2])
def test_cd06_periodic(native_lib, oracle, n, order):
    dx = 2 * np.pi / n
    ls = lines_for(n)
    out = H.plan_apply_lines("cd06", H.params("cd06", n, dx, True), order, 0, 0, ls)
    ref = oracle_lines(lambda l: oracle.cd06(l, dx, periodic=True, order=order), ls)
    assert relerr(out, ref) < tol_for(order, n)


@pytest.mark.parametrize("n", [8, 9, 33])
@pytest.mark.parametrize("bc1,bcn", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_cd06_nonperiodic(native_lib, oracle, n, bc1, bcn):
    dx = 1.0 / (n - 1)
    ls = lines_for(n)
    prm = H.params("cd06", n, dx, False)
    out = H.plan_apply_lines("cd06", prm, 1, bc1, bcn, ls)
    ref = oracle_lines(lambda l: oracle.cd06(l, dx, periodic=False, bc1=bc1, bcn=bcn), ls)
    assert relerr(out, ref) < TOL


@pytest.mark.parametrize("n", [8, 9, 16, 64])
@pytest.mark.parametrize("order", [1, 2])
def test_cd10_periodic(native_lib, oracle, n, order):
    dx = 2 * np.pi / n
    ls = lines_for(n)
    out = H.plan_apply_lines("cd10", H.params("cd10", n, dx, True), order, 0, 0, ls)
    ref = oracle_lines(lambda l: oracle.cd10(l, dx, periodic=True, order=order), ls)
    assert relerr(out, ref) < tol_for(order, n)


@pytest.mark.parametrize("n", [8, 11, 40])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("bc1,bcn", list(itertools.product(BCS, BCS)))
def test_cd10_nonperiodic(native_lib, oracle, n, order, bc1, bcn):
    dx = 1.0 / (n - 1)
    ls = lines_for(n)
    out = H.plan_apply_lines("cd10", H.params("cd10", n, dx, False), order, bc1, bcn, ls)
    ref = oracle_lines(lambda l: oracle.cd10(l, dx, periodic=False, bc1=bc1, bcn=bcn, order=order), ls)
    assert relerr(out, ref) < tol_for(order, n)


@pytest.mark.parametrize("n", [10, 13, 64])
@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("bc1,bcn", list(itertools.product(BCS, BCS)))
def test_cf90(native_lib, oracle, n, periodic, bc1, bcn):
    if periodic and (bc1, bcn) != (0, 0):
        pytest.skip("bc ignored on periodic lines")
    ls = lines_for(n)
    out = H.plan_apply_lines("cf90", H.params("cf90", n, periodic=periodic), 0, bc1, bcn, ls)
    ref = oracle_lines(lambda l: oracle.cf90(l, periodic=periodic, bc1=bc1, bcn=bcn), ls)
    # the CF90 matrix is near-singular at the Nyquist mode (symbol ~2e-3): allow its conditioning
    assert relerr(out, ref) < 2e-12


@pytest.mark.parametrize("n", [9, 16, 64])
@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("bc1,bcn", list(itertools.product(BCS, BCS)))
def test_gaussian(native_lib, oracle, n, periodic, bc1, bcn):
    if periodic and (bc1, bcn) != (0, 0):
        pytest.skip("bc ignored on periodic lines")
    ls = lines_for(n)
    out = H.plan_apply_lines("gaussian", H.params("gaussian", n, periodic=periodic), 0, bc1, bcn, ls)
    ref = oracle_lines(lambda l: oracle.gaussian(l, periodic=periodic, bc1=bc1, bcn=bcn), ls)
    assert relerr(out, ref) < TOL


PER_OPS = ["ddz_E2C", "ddz_C2E", "d2dz2_C2C", "d2dz2_E2E", "InterpZ_E2C", "InterpZ_C2E"]


def stagg_io(op, n):
    nin = n + 1 if op in ("ddz_E2C", "ddz_E2E", "d2dz2_E2E", "InterpZ_E2C") else n
    return nin


@pytest.mark.parametrize("n", [5, 8, 32])
@pytest.mark.parametrize("op", PER_OPS)
def test_stagg_periodic(native_lib, oracle, n, op):
    dx = 1.0 / n
    ls = lines_for(stagg_io(op, n))
    out = H.plan_apply_lines("cd06stagg", H.params("cd06stagg", n, dx, True), H.STAGG[op], 0, 0, ls)
    ref = oracle_lines(lambda l: oracle.stagg(l, n, dx, op, periodic=True, dir=1), ls)
    assert relerr(out, ref) < tol_for(2 if op.startswith("d2") else 1, n)


@pytest.mark.parametrize("n", [8, 17])
@pytest.mark.parametrize("op", list(H.STAGG))
@pytest.mark.parametrize("flags", list(itertools.product([False, True], repeat=4)))
def test_stagg_nonperiodic(native_lib, oracle, n, op, flags):
    topEven, botEven, topSided, botSided = flags
    dx = 1.0 / n
    ls = lines_for(stagg_io(op, n))
    prm = H.params("cd06stagg", n, dx, False, flags)
    out = H.plan_apply_lines("cd06stagg", prm, H.STAGG[op], 0, 0, ls)
    ref = oracle_lines(lambda l: oracle.stagg(l, n, dx, op, periodic=False, topEven=topEven, botEven=botEven,
                                              topSided=topSided, botSided=botSided, dir=1), ls)
    assert relerr(out, ref) < tol_for(2 if op.startswith("d2") else 1, n)


def test_dense_operator_matches_plan(native_lib):
    """The dense restatement (used by the dense path) equals the banded plan."""
    n = 24
    prm = H.params("cd10", n, 0.1, False)
    M = H.dense("cd10", prm, 1, 0, -1)
    ls = lines_for(n)
    out = H.plan_apply_lines("cd10", prm, 1, 0, -1, ls)
    assert relerr(ls @ M.T, out) < 1e-13
