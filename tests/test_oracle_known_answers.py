"""Pin the oracle to the reference's own known answers.

The reference ships no stored output vectors; its tests compare against analytic
functions (tests/test_cd06.F90:27-31, test_cd10.F90:51-81, test_cd10_NP.F90:51-81,
test_cd10_der2.F90:20-32, test_cf90.F90:108-116, test_STAGGcd06.F90:49-56).  Periodic
compact operators act on a Fourier mode exactly through their modified wavenumber /
transfer function, so those symbols pin every interior coefficient and the cyclic
solves to rounding; polynomials the one-sided closures are built to differentiate
exactly pin the boundary rows.
"""
import numpy as np
import pytest

from tests.fields import relerr

pytestmark = []

A06, B06, AL06 = (14 / 9) / 2, (1 / 9) / 4, 1 / 3
A06D2, B06D2, AL06D2 = 12 / 11, (3 / 11) / 4, 2 / 11
A10, B10, C10, AL10, BE10 = (17 / 12) / 2, (101 / 150) / 4, (1 / 100) / 6, 1 / 2, 1 / 20
A10D2, B10D2, C10D2, AL10D2, BE10D2 = 1065 / 1798, (1038 / 899) / 4, (79 / 1798) / 9, 334 / 899, 43 / 1798
CF = dict(alpha=0.66624, beta=0.16688, a=0.99965, b=0.66652, c=0.16674, d=4.0e-5, e=-5.0e-6)
GF = (3565 / 10368, 3091 / 12960, 1997 / 25920, 149 / 12960, 107 / 103680)


def grid(n):
    x = np.arange(n) * 2 * np.pi / n
    return x, x[1] - x[0]


@pytest.mark.parametrize("n", [8, 16, 64, 256])
@pytest.mark.parametrize("k", [1, 3, 7])
def test_cd06_d1_modified_wavenumber(oracle, n, k):
    if k >= n // 2:
        pytest.skip("above Nyquist")
    x, h = grid(n)
    th = k * h
    kmod = (2 * A06 * np.sin(th) + 2 * B06 * np.sin(2 * th)) / (h * (1 + 2 * AL06 * np.cos(th)))
    out = oracle.cd06(np.sin(k * x), h).ravel()
    assert relerr(out, kmod * np.cos(k * x)) < 1e-13


@pytest.mark.parametrize("n", [8, 64])
def test_cd06_d2_completed_symbol(oracle, n):
    x, h = grid(n)
    k = 3
    th = k * h
    sym = -(2 * A06D2 * (1 - np.cos(th)) + 2 * B06D2 * (1 - np.cos(2 * th))) / (h * h * (1 + 2 * AL06D2 * np.cos(th)))
    tol2 = max(1e-13, 50 * np.finfo(float).eps / th ** 2)
    assert relerr(oracle.cd06(np.sin(k * x), h, order=2).ravel(), sym * np.sin(k * x)) < tol2


@pytest.mark.parametrize("n", [8, 9, 32, 256])
@pytest.mark.parametrize("k", [1, 2, 5])
def test_cd10_periodic_symbols(oracle, n, k):
    if k >= n // 2:
        pytest.skip("above Nyquist")
    x, h = grid(n)
    th = k * h
    d1 = (2 * A10 * np.sin(th) + 2 * B10 * np.sin(2 * th) + 2 * C10 * np.sin(3 * th)) / (
        h * (1 + 2 * AL10 * np.cos(th) + 2 * BE10 * np.cos(2 * th)))
    d2 = -(2 * A10D2 * (1 - np.cos(th)) + 2 * B10D2 * (1 - np.cos(2 * th)) + 2 * C10D2 * (1 - np.cos(3 * th))) / (
        h * h * (1 + 2 * AL10D2 * np.cos(th) + 2 * BE10D2 * np.cos(2 * th)))
    f = np.sin(k * x)
    assert relerr(oracle.cd10(f, h).ravel(), d1 * np.cos(k * x)) < 1e-13
    # the second difference cancels by (k h)^2, so FP64 rounding alone is eps / (k h)^2
    tol2 = max(1e-13, 50 * np.finfo(float).eps / th ** 2)
    assert relerr(oracle.cd10(f, h, order=2).ravel(), d2 * f) < tol2


@pytest.mark.parametrize("n", [10, 11, 64])
@pytest.mark.parametrize("k", [1, 4])
def test_cf90_transfer_function(oracle, n, k):
    """test_cf90.F90:108-116 compares against this transfer function."""
    x, h = grid(n)
    th = k * h
    c = CF
    T = (c["a"] + 2 * c["b"] * np.cos(th) + 2 * c["c"] * np.cos(2 * th) + 2 * c["d"] * np.cos(3 * th)
         + 2 * c["e"] * np.cos(4 * th)) / (1 + 2 * c["alpha"] * np.cos(th) + 2 * c["beta"] * np.cos(2 * th))
    f = np.cos(k * x + 0.3)
    assert relerr(oracle.cf90(f).ravel(), T * f) < 1e-13


@pytest.mark.parametrize("n", [9, 64])
def test_gaussian_transfer_function(oracle, n):
    x, h = grid(n)
    k = 2
    th = k * h
    T = GF[0] + sum(2 * GF[j] * np.cos(j * th) for j in range(1, 5))
    f = np.cos(k * x + 0.1)
    assert relerr(oracle.gaussian(f).ravel(), T * f) < 1e-14


STAGG_SYMBOLS = {
    # op: (input on edges?, derivative order, a, b, alpha)
    "ddz_E2C": (True, 1, 63 / 62, (17 / 62) / 3, 9 / 62),
    "ddz_C2E": (False, 1, 63 / 62, (17 / 62) / 3, 9 / 62),
    "InterpZ_E2C": (True, 0, 3 / 4, 1 / 20, 3 / 10),
    "InterpZ_C2E": (False, 0, 3 / 4, 1 / 20, 3 / 10),
    "d2dz2_C2C": (False, 2, 12 / 11, (3 / 11) / 4, 2 / 11),
    "d2dz2_E2E": (True, 2, 12 / 11, (3 / 11) / 4, 2 / 11),
}


@pytest.mark.parametrize("op", sorted(STAGG_SYMBOLS))
@pytest.mark.parametrize("n", [5, 8, 32])
def test_stagg_periodic_symbols(oracle, op, n):
    """test_STAGGcd06.F90:49-56 differentiates sin(2 pi z) + i cos(2 pi z) on periodic edges."""
    onE, order, a, b, al = STAGG_SYMBOLS[op]
    h = 1.0 / n
    ze = np.arange(n + 1) * h
    zc = (np.arange(n) + 0.5) * h
    k = 2 * np.pi
    th = k * h
    src = ze if onE else zc
    outE = op.endswith("2E") or op == "d2dz2_E2E"
    dst = ze if outE else zc
    f = np.sin(k * src)
    if order == 1:
        sym = (2 * a * np.sin(th / 2) + 2 * b * np.sin(1.5 * th)) / (h * (1 + 2 * al * np.cos(th)))
        ex = sym * np.cos(k * dst)
    elif order == 0:
        sym = (2 * a * np.cos(th / 2) + 2 * b * np.cos(1.5 * th)) / (1 + 2 * al * np.cos(th))
        ex = sym * np.sin(k * dst)
    else:
        sym = -(2 * a * (1 - np.cos(th)) + 2 * b * (1 - np.cos(2 * th))) / (h * h * (1 + 2 * al * np.cos(th)))
        ex = sym * np.sin(k * dst)
    out = oracle.stagg(f, n, h, op, periodic=True, dir=1).ravel()
    tol = max(1e-13, 50 * np.finfo(float).eps / th ** 2) if order == 2 else 1e-13
    assert relerr(out, ex) < tol


# ---- boundary closures: polynomial exactness ----
def poly_case(deg, x, order):
    f = x ** deg
    if order == 0:
        return f, x ** deg
    if order == 1:
        return f, (deg * x ** (deg - 1) if deg > 0 else 0 * x)
    return f, (deg * (deg - 1) * x ** (deg - 2) if deg > 1 else 0 * x)


@pytest.mark.parametrize("deg", range(0, 5))
@pytest.mark.parametrize("n", [8, 33])
def test_cd06_nonperiodic_closure_exact(oracle, deg, n):
    x = np.linspace(0, 1, n)
    f, ex = poly_case(deg, x, 1)
    assert np.abs(oracle.cd06(f, x[1], periodic=False).ravel() - ex).max() < 1e-10


@pytest.mark.parametrize("deg", range(0, 5))
@pytest.mark.parametrize("order", [1, 2])
def test_cd10_nonperiodic_closure_exact(oracle, deg, order):
    x = np.linspace(0, 1, 40)
    f, ex = poly_case(deg, x, order)
    assert np.abs(oracle.cd10(f, x[1], periodic=False, order=order).ravel() - ex).max() < 1e-8


@pytest.mark.parametrize("op,degmax", [("ddz_E2C", 3), ("ddz_C2E", 3), ("InterpZ_E2C", 3), ("InterpZ_C2E", 2),
                                       ("ddz_C2C", 4)])
def test_stagg_sided_closure_exact(oracle, op, degmax):
    n = 32
    ze = np.linspace(0, 1, n + 1)
    zc = 0.5 * (ze[1:] + ze[:-1])
    h = ze[1]
    onE = op.endswith("E2C") or op.endswith("E2E")
    outE = op.endswith("2E")
    order = 0 if op.startswith("Interp") else 1
    for deg in range(degmax + 1):
        f = (ze if onE else zc) ** deg
        _, ex = poly_case(deg, ze if outE else zc, order)
        out = oracle.stagg(f, n, h, op, periodic=False, topSided=True, botSided=True, dir=1).ravel()
        assert np.abs(out - ex).max() < 1e-11, (op, deg)


def test_cd10_np_reference_case(oracle):
    """tests/test_cd10_NP.F90: cos(x)cos(y)cos(z) on [0, pi/2]^3 (32^3), bc1 = 1, bcn = -1."""
    n = 32
    x = np.linspace(0, np.pi / 2, n)
    h = x[1]
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    f = np.asfortranarray(np.cos(X) * np.cos(Y) * np.cos(Z))
    for d, (D, E) in enumerate([(X, -np.sin(X) * np.cos(Y) * np.cos(Z)), (Y, -np.cos(X) * np.sin(Y) * np.cos(Z)),
                                (Z, -np.cos(X) * np.cos(Y) * np.sin(Z))], start=1):
        out = oracle.cd10(f, h, periodic=False, bc1=1, bcn=-1, dir=d)
        assert np.abs(out - E).max() < 1e-9


def test_error_codes_match_reference(oracle):
    from oracle.oracle import OracleError

    x = np.zeros(5)
    with pytest.raises(OracleError) as e:
        oracle.cd06(x, 0.1, periodic=True)
    assert e.value.code == 3
    with pytest.raises(OracleError) as e:
        oracle.cd10(np.zeros(7), 0.1)
    assert e.value.code == 2
    with pytest.raises(OracleError) as e:
        oracle.cf90(np.zeros(9))
    assert e.value.code == 7
    with pytest.raises(OracleError) as e:
        oracle.cd10(np.zeros(16), 0.1, periodic=False, bc1=2)
    assert e.value.code == 324
