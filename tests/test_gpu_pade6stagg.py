"""Pade6stagg (PadeDerOps.F90) against the oracle's cd06stagg restatement (GPU).

Every (bot, top) pair in {-1, 0, 1}^2 and every operation, REAL and CMPLX, device and host
buffers.  The expected cd06stagg configuration of each pair is written out here from
PadeDerOps.F90:92-110 (der<Top><Bot>: isTopEven, isBotEven, isTopSided, isBotSided) and
its selection from PadeDerOps.F90:146-995; pairs without an operator give zero output.
Tolerances as tests/test_gpu_parity.py: 1e-12 normwise, second derivatives at the FP64
conditioning of the second difference.
"""
import numpy as np
import pytest

import padeops_gb300 as P
from oracle import spectral_oracle as SO
from tests.fields import relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
EPS = np.finfo(np.float64).eps

# (bot, top) -> (isTopEven, isBotEven, isTopSided, isBotSided) of the selected object
VARIANT = {(-1, -1): (False, False, False, False),  # derOO
           (-1, 0): (False, False, True, False),    # derSO
           (-1, 1): (True, False, False, False),    # derEO
           (0, -1): (False, False, False, True),    # derOS
           (0, 0): (True, True, True, True),        # derSS
           (0, 1): (True, True, False, True),       # derES
           (1, -1): (False, True, False, False),    # derOE
           (1, 0): (True, True, True, False),       # derSE
           (1, 1): (True, True, False, False)}      # derEE
# facade op -> (cd06stagg procedure, input on edges, output on edges)
OPS = {"ddz_C2E": ("ddz_C2E", False, True), "ddz_E2C": ("ddz_E2C", True, False),
       "interpz_C2E": ("InterpZ_C2E", False, True), "interpz_E2C": ("InterpZ_E2C", True, False),
       "d2dz2_C2C": ("d2dz2_C2C", False, False), "d2dz2_E2E": ("d2dz2_E2E", True, True)}


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def to_host(t):
    return np.asfortranarray(t.cpu().numpy().T)


def field(shape, seed, cplx):
    rng = np.random.default_rng(seed)
    z = np.linspace(0, 1, shape[2])[None, None, :]
    f = np.cos(3 * z + rng.standard_normal(shape[:2])[:, :, None]) + 0.05 * rng.standard_normal(shape)
    if cplx:
        f = f + 1j * (np.sin(2 * z) + 0.05 * rng.standard_normal(shape))
    return np.asfortranarray(f)


def tol(op, f, ref, dz):
    if not op.startswith("d2"):
        return 1e-12
    return max(1e-12, 50 * EPS * np.abs(f).max() / (dz * dz * max(np.abs(ref).max(), 1e-300)))


def expected(oracle, name, f, nz, dz, bot, top, periodic):
    proc = OPS[name][0]
    if periodic:
        flags = dict(periodic=True)
    else:
        if name.startswith("d2") and (bot == 0 or top == 0):
            return None  # the reference sets output = 0
        te, be, ts, bs = VARIANT[(bot, top)]
        flags = dict(periodic=False, topEven=te, botEven=be, topSided=ts, botSided=bs)
    if np.iscomplexobj(f):
        return oracle.stagg(np.ascontiguousarray(f.real), nz, dz, proc, **flags) + \
            1j * oracle.stagg(np.ascontiguousarray(f.imag), nz, dz, proc, **flags)
    return oracle.stagg(f, nz, dz, proc, **flags)


@pytest.mark.parametrize("cplx", [False, True], ids=["real", "cmplx"])
@pytest.mark.parametrize("name", list(OPS))
def test_nine_boundary_pairs(oracle, name, cplx):
    nz, n1, n2 = 48, 6, 5
    dz = 1.0 / nz
    p = P.Pade6stagg()
    assert p.init(nz, dz, P.PadeDerOps.cd06, False) == 0
    _, e_in, e_out = OPS[name]
    f = field((n1, n2, nz + (1 if e_in else 0)), 3, cplx)
    oshape = (n1, n2, nz + (1 if e_out else 0))
    dt = torch.complex128 if cplx else torch.float64
    for bot in (-1, 0, 1):
        for top in (-1, 0, 1):
            ref = expected(oracle, name, f, nz, dz, bot, top, False)
            out = torch.full(tuple(reversed(oshape)), 7.0, dtype=dt, device="cuda")
            getattr(p, name)(to_dev(f), out, bot, top)
            torch.cuda.synchronize()
            got = to_host(out)
            if ref is None:
                assert np.all(got == 0), (bot, top)
            else:
                assert relerr(got, ref) < tol(name, f, ref, dz), (bot, top)
    # host buffers, one pair, through the named C entry point
    ref = expected(oracle, name, f, nz, dz, 1, -1, False)
    out = np.zeros(oshape, dtype=f.dtype, order="F")
    getattr(p, name)(f, out, 1, -1)
    assert relerr(out, ref) < tol(name, f, ref, dz)
    p.destroy()


@pytest.mark.parametrize("name", list(OPS))
def test_periodic_ignores_boundary_codes(oracle, name):
    nz, n1, n2 = 64, 4, 3
    dz = 2 * np.pi / nz
    p = P.Pade6stagg()
    assert p.init(nz, dz, P.PadeDerOps.cd06, True) == 0
    _, e_in, e_out = OPS[name]
    f = field((n1, n2, nz + (1 if e_in else 0)), 5, False)
    if e_in:
        f[:, :, -1] = f[:, :, 0]  # periodic edge field
    ref = expected(oracle, name, f, nz, dz, 0, 0, True)
    for bot, top in ((0, 0), (-1, 1), (5, 5)):
        out = np.zeros((n1, n2, nz + (1 if e_out else 0)), order="F")
        getattr(p, name)(f, out, bot, top)
        assert relerr(out, ref) < tol(name, f, ref, dz), (bot, top)


def test_modified_wavenumbers_and_poincare_constant():
    nz, dz = 32, 2 * np.pi / 32
    p = P.Pade6stagg()
    assert p.init(nz, dz, P.PadeDerOps.cd06, True) == 0
    k = SO.GetWaveNums(nz, dz)
    assert np.allclose(p.getModifiedWavenumbers(k), SO.getmodCD06stagg(k, dz), rtol=1e-15, atol=0)
    assert p.getApproxPoincareConstant() == 1.0 / np.sqrt(10.0)


def test_invalid_codes_give_zero_output(oracle):
    nz, dz = 16, 1.0 / 16
    p = P.Pade6stagg()
    assert p.init(nz, dz, P.PadeDerOps.cd06, False) == 0
    f = field((3, 2, nz), 1, False)
    out = np.ones((3, 2, nz + 1), order="F")
    p.ddz_C2E(f, out, 2, -1)  # bot outside {-1, 0, 1}: case default, output = 0
    assert np.all(out == 0)


# ---- the second-order scheme (fd02: staggOps.F90 through PadeDerOps.F90's fd02 branches) ----
FD02_INDEX = {"ddz_C2E": 0, "ddz_E2C": 1, "interpz_C2E": 2, "interpz_E2C": 3, "d2dz2_C2C": 4, "d2dz2_E2E": 5}


@pytest.mark.parametrize("periodic", [False, True], ids=["walls", "periodic"])
@pytest.mark.parametrize("cplx", [False, True], ids=["real", "cmplx"])
@pytest.mark.parametrize("name", list(OPS))
def test_fd02_every_code_pair(name, cplx, periodic):
    from oracle import fd02_oracle as FO

    nz, n1, n2 = 40, 5, 4
    dz = 1.0 / nz
    p = P.Pade6stagg()
    assert p.init(nz, dz, P.PadeDerOps.fd02, periodic) == 0
    _, e_in, e_out = OPS[name]
    f = field((n1, n2, nz + (1 if e_in else 0)), 7, cplx)
    oshape = (n1, n2, nz + (1 if e_out else 0))
    dt = torch.complex128 if cplx else torch.float64
    pairs = [(b, t) for b in (-1, 0, 1) for t in (-1, 0, 1)] + [(2, 1), (-1, 5)]
    for bot, top in pairs:
        ref = FO.apply(FD02_INDEX[name], f, dz, periodic, bot, top)
        out = torch.full(tuple(reversed(oshape)), 7.0, dtype=dt, device="cuda")
        getattr(p, name)(to_dev(f), out, bot, top)
        torch.cuda.synchronize()
        got = to_host(out)
        if not np.any(ref):
            assert np.all(got == 0), (bot, top)
        else:
            assert relerr(got, ref) < tol(name, f, ref, dz), (bot, top)
    # host buffers through the named C entry point
    ref = FO.apply(FD02_INDEX[name], f, dz, periodic, 1, -1)
    out = np.zeros(oshape, dtype=f.dtype, order="F")
    getattr(p, name)(f, out, 1, -1)
    assert relerr(out, ref) < tol(name, f, ref, dz) if np.any(ref) else np.all(out == 0)
    p.destroy()


# ---- Fourier collocation in z (periodic; spectral.F90's z operators) ----
@pytest.mark.parametrize("nz", [32, 256])
@pytest.mark.parametrize("cplx", [False, True], ids=["real", "cmplx"])
@pytest.mark.parametrize("name", list(OPS))
def test_fourier_collocation(name, cplx, nz):
    n1, n2 = 6, 5
    dz = 2 * np.pi / nz
    p = P.Pade6stagg()
    assert p.init(nz, dz, P.PadeDerOps.fourierColl, True) == 0
    _, e_in, e_out = OPS[name]
    rng = np.random.default_rng(nz + 3 * cplx)
    z = np.arange(nz + (1 if e_in else 0)) * dz
    f = np.cos(3 * z)[None, None, :] + 0.3 * np.sin(7 * z + rng.standard_normal((n1, n2, 1))) + \
        0.01 * rng.standard_normal((n1, n2, z.size))
    if cplx:
        f = f + 1j * (np.sin(2 * z)[None, None, :] + 0.01 * rng.standard_normal((n1, n2, z.size)))
    f = np.asfortranarray(f)
    ref = SO.fourier_coll(FD02_INDEX[name], f, nz, dz)
    dt = torch.complex128 if cplx else torch.float64
    out = torch.zeros(tuple(reversed(ref.shape)), dtype=dt, device="cuda")
    for bot, top in ((0, 0), (-1, 1), (9, 9)):  # periodic: the codes are ignored
        getattr(p, name)(to_dev(f), out, bot, top)
        torch.cuda.synchronize()
        assert relerr(to_host(out), ref) < 1e-12, (bot, top)
    assert np.allclose(p.getModifiedWavenumbers(SO.GetWaveNums(nz, dz)), SO.GetWaveNums(nz, dz), rtol=0, atol=0)
    assert p.getApproxPoincareConstant() == 1.0 / np.sqrt(12.0)
