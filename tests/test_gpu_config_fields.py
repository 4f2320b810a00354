"""The benchmark configurations' own fields through the CUDA path (GPU).

Config 1: the plain CD06 periodic first derivative ddx / ddy / ddz (cd06%dd1/dd2/dd3,
cd06.F90:775-839) on a 64^3 FP64 grid over [0, 2pi)^3, u = sum of 32 Fourier modes with
integer wavevectors |k_i| <= 16 (numpy PCG64 seed 1), amplitudes N(0,1)|k|^-5/6 and
random phases.  Checked against the oracle (1e-12 normwise) and against the analytic
derivative: the CUDA path's error there must be the scheme's own truncation error, i.e.
equal to the oracle's error against the analytic derivative to within 1e-12 of the
derivative's maximum (the modes reach k dx = pi/2, where CD06's modified wavenumber is 1 %
low, so the truncation error itself is ~1e-2).

Config 2's field (256^3, 32 modes |k_i| <= 64, tanh z profile, seed 2) through the nine
operator applications of the benchmark step is compared with the oracle by bench.py
itself (parity_relerr of its JSON line).
"""
import numpy as np
import pytest

import padeops_gb300 as P
from tests.fields import random_modes, relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def to_host(t):
    return np.asfortranarray(t.cpu().numpy().T)


def test_config1_cd06_periodic_first_derivatives(oracle):
    n = 64
    f, grad = random_modes(n, 32, 16, 1, gradient=True)
    dx = 2 * np.pi / n
    c = P.cd06()
    assert c.init(n, dx, True, 0, 0) == 0
    fd = to_dev(f)
    for d, fn in ((1, c.dd1), (2, c.dd2), (3, c.dd3)):
        od = torch.empty_like(fd)
        fn(fd, od, n, n)
        torch.cuda.synchronize()
        got = to_host(od)
        ref = oracle.cd06(f, dx, periodic=True, dir=d)
        assert relerr(got, ref) < 1e-12, d
        exact = grad[d - 1]
        scale = np.abs(exact).max()
        e_gpu = np.abs(got - exact).max() / scale
        e_ref = np.abs(ref - exact).max() / scale
        assert abs(e_gpu - e_ref) < 1e-12, d
        assert 1e-4 < e_ref < 5e-2, (d, e_ref)  # CD06 truncation at k dx <= pi/2
    # host buffers (staged by the library) give the same answer
    out = np.zeros_like(f, order="F")
    c.dd1(f, out, n, n)
    assert relerr(out, oracle.cd06(f, dx, periodic=True, dir=1)) < 1e-12
