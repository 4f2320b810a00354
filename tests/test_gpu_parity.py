"""Parity of the CUDA path with the oracle (GPU).

Every family, boundary combination, direction and arithmetic path runs through the C
ABI on seeded fields and is compared with the oracle's restatement of the reference on
the same input.  Tolerances (normwise relative, max|a-b|/max|b|):
  FP64 paths (double-float and native)  1e-12 for first derivatives and filters (CF90
      included, white-noise input too: the double-float path runs CF90 in residual form,
      f - A^-1 ((A - B) f), whose right-hand side is ~1e-4 of f, so the solve's amplification
      at the Nyquist mode acts on a small quantity; measured worst case 2.2e-13 over n = 40,
      64, 256, periodic and all nine bc pairs, the oracle's own FP64 level);
      second derivatives allow the FP64 conditioning of the second difference,
      50*eps*max|f|/(h^2 max|f''|), when that is larger.
  FP32 path                             3e-5 (5e-4 for cf90, whose matrix is near
      singular at the Nyquist mode)
"""
import itertools

import numpy as np
import pytest

import padeops_gb300 as P
from padeops_gb300 import _lib as L
from tests.fields import random_modes, relerr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
BCS = [0, 1, -1]
EPS = np.finfo(np.float64).eps


def to_dev(a, dtype=torch.float64):
    """Fortran-ordered numpy array -> CUDA tensor with the same memory order."""
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).to("cuda", dtype)


def to_host(t, shape):
    return np.asfortranarray(t.cpu().numpy().T.reshape(shape, order="F"))


def other_extents(shape, dir):
    s = list(shape)
    del s[dir - 1]
    return s


def field(shape, seed):
    rng = np.random.default_rng(seed)
    n1, n2, n3 = shape
    x = [np.linspace(0, 2 * np.pi, s, endpoint=False) for s in shape]
    X, Y, Z = np.meshgrid(*x, indexing="ij")
    f = np.sin(2 * X + 0.3) * np.cos(Y - 0.2) + 0.5 * np.cos(3 * Z + X) + 0.1 * rng.standard_normal(shape)
    return np.asfortranarray(f)


def tol64(order, f, ref, h):
    if order < 2:
        return 1e-12
    cond = 50 * EPS * np.abs(f).max() / (h * h * max(np.abs(ref).max(), 1e-300))
    return max(1e-12, cond)


def run(obj, opcode, dir, f, out_shape, bc1=0, bcn=0, path=L.PATH_DF, dtype=torch.float64):
    fd = to_dev(f, dtype)
    od = torch.empty(tuple(reversed(out_shape)), dtype=dtype, device="cuda")
    na, nb = other_extents(f.shape, dir)
    obj.apply(opcode, dir, fd, od, na, nb, bc1, bcn, path)
    torch.cuda.synchronize()
    return to_host(od, out_shape).astype(np.float64)


PATHS = [L.PATH_DF, L.PATH_NATIVE]


def shape_for(n, dir, other=(12, 10)):
    s = list(other)
    s.insert(dir - 1, n)
    return tuple(s)


@pytest.mark.parametrize("dir", [1, 2, 3])
@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("n,periodic", [(16, True), (64, True), (6, True), (33, False), (8, False)])
def test_cd06(oracle, dir, path, n, periodic):
    dx = 2 * np.pi / n if periodic else 1.0 / (n - 1)
    o = P.cd06()
    assert o.init(n, dx, periodic, 0, 0) == 0
    shape = shape_for(n, dir)
    f = field(shape, 1)
    for order in ([1, 2] if periodic else [1]):
        out = run(o, order, dir, f, shape, path=path)
        ref = oracle.cd06(f, dx, periodic=periodic, order=order, dir=dir)
        assert relerr(out, ref) < tol64(order, f, ref, dx)


@pytest.mark.parametrize("dir", [1, 2, 3])
@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("n", [8, 16, 40, 256])
def test_cd10_periodic(oracle, dir, path, n):
    dx = 2 * np.pi / n
    o = P.cd10()
    assert o.init(n, dx, True) == 0
    shape = shape_for(n, dir, (6, 5) if n > 64 else (12, 10))
    f = field(shape, 2)
    for order in (1, 2):
        out = run(o, order, dir, f, shape, path=path)
        ref = oracle.cd10(f, dx, periodic=True, order=order, dir=dir)
        assert relerr(out, ref) < tol64(order, f, ref, dx)


@pytest.mark.parametrize("bc1,bcn", list(itertools.product(BCS, BCS)))
@pytest.mark.parametrize("dir", [1, 3])
@pytest.mark.parametrize("n", [8, 27, 64])
def test_cd10_nonperiodic(oracle, bc1, bcn, dir, n):
    dx = 1.0 / (n - 1)
    o = P.cd10()
    assert o.init(n, dx, False) == 0
    shape = shape_for(n, dir)
    f = field(shape, 3)
    for order in (1, 2):
        for path in PATHS:
            out = run(o, order, dir, f, shape, bc1, bcn, path)
            ref = oracle.cd10(f, dx, periodic=False, bc1=bc1, bcn=bcn, order=order, dir=dir)
            assert relerr(out, ref) < tol64(order, f, ref, dx), (order, path)


@pytest.mark.parametrize("fam", ["cd06", "cd10"])
@pytest.mark.parametrize("dir", [1, 2, 3])
@pytest.mark.parametrize("n", [32, 48, 80, 96, 160, 224])
def test_periodic_whole_chunks(oracle, fam, dir, n):
    """Periodic lines of whole chunks for the half-chunk line kernel: 1, 3, 5 and 7 chunks of
    32 rows (one lane per line, idle lanes in the scan groups) and 3 and 5 chunks of 16 rows
    (lengths that are not multiples of 32), over a ragged 7 x 5 set of lines."""
    dx = 2 * np.pi / n
    o = getattr(P, fam)()
    assert o.init(n, dx, True) == 0
    shape = shape_for(n, dir, (7, 5))
    f = field(shape, 5)
    for order in (1, 2):
        out = run(o, order, dir, f, shape)
        ref = getattr(oracle, fam)(f, dx, periodic=True, order=order, dir=dir)
        assert relerr(out, ref) < tol64(order, f, ref, dx), order


@pytest.mark.parametrize("bc1,bcn", list(itertools.product(BCS, BCS)))
@pytest.mark.parametrize("dir", [1, 3])
@pytest.mark.parametrize("n", [64, 96, 160, 256])
def test_banded_whole_chunks(oracle, bc1, bcn, dir, n):
    """Non-periodic lines of 2, 3, 5 and 8 chunks of 32 rows (the banded half-chunk kernel for
    the derivatives: the leading and the last lanes with their own tables, the interior lanes
    on the shared pattern; cf90 stays on k_line), cd10 d1 / d2 and cf90, every bc pair, a
    ragged set of lines."""
    shape = shape_for(n, dir, (7, 5) if n > 64 else (12, 10))
    f = field(shape, 6)
    dx = 1.0 / (n - 1)
    o = P.cd10()
    assert o.init(n, dx, False) == 0
    for order in (1, 2):
        out = run(o, order, dir, f, shape, bc1, bcn)
        ref = oracle.cd10(f, dx, periodic=False, bc1=bc1, bcn=bcn, order=order, dir=dir)
        assert relerr(out, ref) < tol64(order, f, ref, dx), order
    c = P.cf90()
    assert c.init(n, False) == 0
    out = run(c, 0, dir, f, shape, bc1, bcn)
    assert relerr(out, oracle.cf90(f, periodic=False, bc1=bc1, bcn=bcn, dir=dir)) < 1e-12


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("bc1,bcn", list(itertools.product(BCS, BCS)))
@pytest.mark.parametrize("dir", [1, 2, 3])
def test_cf90(oracle, periodic, bc1, bcn, dir):
    if periodic and (bc1, bcn) != (0, 0):
        pytest.skip("bc ignored on periodic lines")
    n = 40
    o = P.cf90()
    assert o.init(n, periodic) == 0
    shape = shape_for(n, dir)
    f = field(shape, 4)
    for path in PATHS:
        out = run(o, 0, dir, f, shape, bc1, bcn, path)
        ref = oracle.cf90(f, periodic=periodic, bc1=bc1, bcn=bcn, dir=dir)
        assert relerr(out, ref) < 1e-12, path


@pytest.mark.parametrize("n", [64, 256])
@pytest.mark.parametrize("periodic,bc1,bcn", [(True, 0, 0)] + [(False, a, b) for a in BCS for b in BCS])
def test_cf90_white_noise(oracle, n, periodic, bc1, bcn):
    """Pure white noise (the CF90 matrix's worst case) on every path at 1e-12."""
    o = P.cf90()
    assert o.init(n, periodic) == 0
    rng = np.random.default_rng(n + 3 * bc1 + bcn)
    for dir in (1, 3):
        shape = shape_for(n, dir, (8, 6))
        f = np.asfortranarray(rng.standard_normal(shape))
        ref = oracle.cf90(f, periodic=periodic, bc1=bc1, bcn=bcn, dir=dir)
        for path in PATHS:
            assert relerr(run(o, 0, dir, f, shape, bc1, bcn, path), ref) < 1e-12, (dir, path)


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("bc1,bcn", [(0, 0), (1, -1), (-1, 1)])
@pytest.mark.parametrize("dir", [1, 2, 3])
def test_gaussian(oracle, periodic, bc1, bcn, dir):
    n = 24
    o = P.gaussian()
    assert o.init(n, periodic) == 0
    shape = shape_for(n, dir)
    f = field(shape, 5)
    for path in PATHS:
        out = run(o, 0, dir, f, shape, bc1, bcn, path)
        ref = oracle.gaussian(f, periodic=periodic, bc1=bc1, bcn=bcn, dir=dir)
        assert relerr(out, ref) < 1e-12


STAGG_PER = ["ddz_E2C", "ddz_C2E", "d2dz2_C2C", "d2dz2_E2E", "InterpZ_E2C", "InterpZ_C2E"]
ONE = ("ddz_E2C", "ddz_E2E", "d2dz2_E2E", "InterpZ_E2C")
OUTE = ("ddz_C2E", "ddz_E2E", "d2dz2_E2E", "InterpZ_C2E")


def stagg_shapes(n, op, n1=10, n2=9):
    nin = n + 1 if op in ONE else n
    nout = n + 1 if op in OUTE else n
    return (n1, n2, nin), (n1, n2, nout)


@pytest.mark.parametrize("op", STAGG_PER)
@pytest.mark.parametrize("n", [5, 32, 128, 257])
def test_stagg_periodic(oracle, op, n):
    dx = 1.0 / n
    o = P.cd06stagg()
    assert o.init(n, dx) == 0
    sin, sout = stagg_shapes(n, op)
    f = field(sin, 6)
    f[:, :, -1] = f[:, :, 0] if op in ONE else f[:, :, -1]  # periodic edge data: f(n+1) = f(1)
    ref = oracle.stagg(f, n, dx, op, periodic=True)
    for path in PATHS:
        out = run(o, L.STAGG_OPS.index(op), 3, f, sout, path=path)
        assert relerr(out, ref) < tol64(2 if op.startswith("d2") else 1, f, ref, dx), path


@pytest.mark.parametrize("op", ["ddz_E2C", "InterpZ_E2C"])
@pytest.mark.parametrize("n", [16, 64, 96])
def test_stagg_periodic_edge_point_as_given(oracle, op, n):
    """Periodic edges to cells read the (n+1)-th edge as stored (cd06stagg.F90:319, 544),
    whether or not it repeats the first: the line kernels (n a multiple of 32) and the
    generic chunked kernel (n = 16) alike."""
    dx = 1.0 / n
    o = P.cd06stagg()
    assert o.init(n, dx) == 0
    sin, sout = stagg_shapes(n, op)
    f = field(sin, 12)
    assert np.abs(f[:, :, -1] - f[:, :, 0]).max() > 0.1
    ref = oracle.stagg(f, n, dx, op, periodic=True)
    out = run(o, L.STAGG_OPS.index(op), 3, f, sout, path=L.PATH_DF)
    assert relerr(out, ref) < tol64(1, f, ref, dx)


@pytest.mark.parametrize("op", list(L.STAGG_OPS))
@pytest.mark.parametrize("flags", [(False, False, False, False), (True, True, False, False),
                                   (True, False, True, True), (False, True, True, False), (False, False, True, True)])
def test_stagg_nonperiodic(oracle, op, flags):
    n = 48
    dx = 1.0 / n
    o = P.cd06stagg()
    assert o.init(n, dx, *flags) == 0
    sin, sout = stagg_shapes(n, op)
    f = field(sin, 7)
    ref = oracle.stagg(f, n, dx, op, periodic=False, topEven=flags[0], botEven=flags[1], topSided=flags[2],
                       botSided=flags[3])
    for path in PATHS:
        out = run(o, L.STAGG_OPS.index(op), 3, f, sout, path=path)
        assert relerr(out, ref) < tol64(2 if op.startswith("d2") else 1, f, ref, dx), path


def test_named_entry_points_and_complex(oracle):
    """The reference-named procedures, REAL and CMPLX overloads, device and host buffers."""
    n1, n2, n = 10, 8, 32
    dz = 1.0 / n
    s = P.cd06stagg()
    assert s.init(n, dz) == 0
    rng = np.random.default_rng(8)
    fE = np.asfortranarray(rng.standard_normal((n1, n2, n + 1)) + 1j * rng.standard_normal((n1, n2, n + 1)))
    fE[:, :, -1] = fE[:, :, 0]
    dfC = torch.empty((n, n2, n1), dtype=torch.complex128, device="cuda")
    s.ddz_E2C(to_dev(fE, torch.complex128), dfC, n1, n2)
    got = to_host(dfC, (n1, n2, n))
    ref = oracle.stagg(fE.real, n, dz, "ddz_E2C") + 1j * oracle.stagg(fE.imag, n, dz, "ddz_E2C")
    assert relerr(got, ref) < 1e-12
    # host numpy buffers (staged by the library) through the same entry
    out = np.zeros((n1, n2, n), dtype=np.complex128, order="F")
    s.ddz_E2C(fE, out, n1, n2)
    assert relerr(out, ref) < 1e-12
    # cd10 named entries with host arrays
    c = P.cd10()
    assert c.init(n, 2 * np.pi / n, True) == 0
    f = field((n, n1, n2), 9)
    df = np.zeros_like(f, order="F")
    c.dd1(f, df, n1, n2)
    assert relerr(df, oracle.cd10(f, 2 * np.pi / n, dir=1)) < 1e-12
    # cf90 filter3 on complex data (CMPLX overload)
    cf = P.cf90()
    assert cf.init(n, False) == 0
    g = np.asfortranarray(rng.standard_normal((n1, n2, n)) + 1j * rng.standard_normal((n1, n2, n)))
    gf = np.zeros_like(g, order="F")
    cf.filter3(g, gf, n1, n2, 0, 0)
    refc = oracle.cf90(g.real, periodic=False, dir=3) + 1j * oracle.cf90(g.imag, periodic=False, dir=3)
    assert relerr(gf, refc) < 1e-12  # white-noise input


@pytest.mark.parametrize("fam", ["cd10", "cf90", "cd06"])
def test_fp32_path(oracle, fam):
    n = 64
    shape = (n, 16, 12)
    f = field(shape, 10)
    if fam == "cd10":
        o = P.cd10(); o.init(n, 2 * np.pi / n, True)
        ref = oracle.cd10(f, 2 * np.pi / n)
        opc, tol = 1, 3e-5
    elif fam == "cd06":
        o = P.cd06(); o.init(n, 1.0 / (n - 1), False)
        ref = oracle.cd06(f, 1.0 / (n - 1), periodic=False)
        opc, tol = 1, 3e-5
    else:
        o = P.cf90(); o.init(n, True)
        ref = oracle.cf90(f)
        opc, tol = 0, 5e-4
    for dir in (1, 3):
        r = ref if dir == 1 else None
        if dir == 3:
            g = np.asfortranarray(np.transpose(f, (1, 2, 0)))
            r = np.transpose(ref, (1, 2, 0))
            out = run(o, opc, 3, g, g.shape, path=L.PATH_FP32, dtype=torch.float32)
        else:
            out = run(o, opc, 1, f, shape, path=L.PATH_FP32, dtype=torch.float32)
        assert relerr(out, r) < tol


def test_bench_scale_fields(oracle):
    """256^2 x 64 slab of the benchmark field, all three directions of cd10 (d1, d2) and cf90."""
    n = 256
    f = random_modes((n, n, 24), 32, 64, seed=2)
    dx = 2 * np.pi / n
    c = P.cd10()
    assert c.init(n, dx, True) == 0
    cf = P.cf90()
    assert cf.init(n, True) == 0
    for dir in (1, 2):
        for order in (1, 2):
            out = run(c, order, dir, f, f.shape)
            ref = oracle.cd10(f, dx, order=order, dir=dir)
            assert relerr(out, ref) < tol64(order, f, ref, dx)
        out = run(cf, 0, dir, f, f.shape)
        assert relerr(out, oracle.cf90(f, dir=dir)) < 1e-12


@pytest.mark.parametrize("amp", [1e-300, 1e-200, 1e-30, 1e30, 1e200, 1e300])
def test_double_float_path_is_range_free(oracle, amp):
    """Each line is scaled by a power of two before the double-float split, so any FP64
    magnitude keeps full relative accuracy, along every direction."""
    n = 16
    c = P.cd10()
    assert c.init(n, 0.1, True) == 0
    z = P.cf90()
    assert z.init(n, False) == 0
    f = field((n, n, n), 9) * amp
    f[:, 2, 3] *= 1e-80  # a line far below the others keeps its own relative accuracy
    for dir in (1, 2, 3):
        out = run(c, 1, dir, f, f.shape)
        ref = oracle.cd10(f, 0.1, order=1, dir=dir)
        assert relerr(out, ref) < 1e-12, dir
        out = run(z, 0, dir, f, f.shape)
        assert relerr(out, oracle.cf90(f, periodic=False, dir=dir)) < 1e-12, dir
    out = run(c, 1, 1, f, f.shape)
    ref = oracle.cd10(f, 0.1, order=1, dir=1)
    assert relerr(out[:, 2, 3], ref[:, 2, 3]) < 1e-12


def test_range_flag_for_non_finite_input(oracle):
    """A NaN or infinity in a line raises PADE_ERANGE on host-buffer calls."""
    n = 16
    c = P.cd10()
    assert c.init(n, 0.1, True) == 0
    f = np.zeros((n, 4, 4), order="F")
    f[3, 1, 1] = np.inf
    df = np.zeros_like(f, order="F")
    with pytest.raises(L.PadeError) as e:
        c.dd1(f, df, 4, 4)
    assert e.value.code == L.PADE_ERANGE


def test_empty_line_sets_are_no_ops(native_lib):
    """No lines (na or nb = 0): success and nothing done, as the reference's loops over
    empty arrays; null field pointers are accepted then.  Negative counts stay errors."""
    import ctypes

    h = ctypes.c_void_p()
    assert native_lib.pade_cd10_init(ctypes.byref(h), 32, 0.1, 1, 0, 0) == 0
    try:
        for na, nb in ((0, 4), (4, 0), (0, 0)):
            assert native_lib.pade_apply(h, 1, 1, 0, None, None, na, nb, 0, 0, L.PATH_DF, None) == 0
            assert native_lib.pade_apply_noalloc(h, 1, 2, 0, None, None, na, nb, 0, 0, None) == 0
        assert native_lib.pade_apply(h, 1, 1, 0, None, None, -1, 4, 0, 0, L.PATH_DF, None) == L.PADE_EINVAL
        assert native_lib.pade_apply(h, 1, 1, 0, None, None, 4, 4, 0, 0, L.PATH_DF, None) == L.PADE_EINVAL
        c = P.cd10()
        assert c.init(32, 0.1, True) == 0
        f = np.zeros((32, 0, 3), order="F")
        df = np.zeros_like(f, order="F")
        c.dd1(f, df, 0, 3)
    finally:
        native_lib.pade_destroy(h)


def test_reference_error_codes():
    c = P.cd10()
    assert c.init(7, 0.1, True) == L.PADE_EREF_NONPERIODIC_N
    assert c.init(16, 0.1, False) == 0
    f = np.zeros((16, 2, 2), order="F")
    with pytest.raises(L.PadeError) as e:
        c.dd1(f, np.zeros_like(f), 2, 2, 3, 0)
    assert e.value.code == L.PADE_EREF_BC
    d = P.cd06()
    assert d.init(16, 0.1, False) == 0
    with pytest.raises(L.PadeError) as e:
        d.d2d1(f, np.zeros_like(f), 2, 2)
    assert e.value.code == L.PADE_ENOTSUP
    s = P.cd06stagg()
    assert s.init(4, 0.1) == L.PADE_EREF_STAGG_N
