"""Generate tests/golden/golden.npz: the oracle's answers on the reference tests' own inputs.

The reference stores no output vectors and its Fortran cannot be built here, so the
fixtures are (a) the inputs of the reference's test programs, reduced to one line each
(their fields are separable), with the analytic answers those programs compare against
and the oracle's output on them, and (b) a few seeded lines per operator family,
direction-independent, with the oracle's output.  tests/test_golden.py checks that the
oracle still reproduces the fixtures (CPU) and that the CUDA path matches them (GPU).

    python tests/golden/make_golden.py        # rewrites tests/golden/golden.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def line3(v):
    """A 1-D profile as an (n, 1, 1) Fortran array (lines along x)."""
    return np.asfortranarray(np.asarray(v, dtype=np.float64).reshape(-1, 1, 1))


def main():
    O.build()
    g = {}
    # tests/test_cd06.F90:9-31: nx = 256 periodic, f = sin(x), df = cos(x)
    n = 256
    h = 2 * np.pi / n
    x = np.arange(n) * h
    g["cd06_p256_f"] = np.sin(x)
    g["cd06_p256_exact"] = np.cos(x)
    g["cd06_p256_oracle"] = O.cd06(line3(np.sin(x)), h, periodic=True).ravel()
    # tests/test_cd10.F90:9-81: nx = 32 periodic, f = sin(x): d1 cos(x), d2 -sin(x)
    n = 32
    h = 2 * np.pi / n
    x = np.arange(n) * h
    g["cd10_p32_f"] = np.sin(x)
    g["cd10_p32_d1_exact"] = np.cos(x)
    g["cd10_p32_d2_exact"] = -np.sin(x)
    g["cd10_p32_d1_oracle"] = O.cd10(line3(np.sin(x)), h, periodic=True, order=1).ravel()
    g["cd10_p32_d2_oracle"] = O.cd10(line3(np.sin(x)), h, periodic=True, order=2).ravel()
    # tests/test_cd10_NP.F90:9-81: nx = 32 non-periodic, dx = 2 pi/(n-1), f = cos(x)
    h = 2 * np.pi / (n - 1)
    x = np.arange(n) * h
    g["cd10_np32_f"] = np.cos(x)
    g["cd10_np32_d1_exact"] = -np.sin(x)
    g["cd10_np32_d2_exact"] = -np.cos(x)
    g["cd10_np32_d1_oracle"] = O.cd10(line3(np.cos(x)), h, periodic=False, order=1).ravel()
    g["cd10_np32_d2_oracle"] = O.cd10(line3(np.cos(x)), h, periodic=False, order=2).ravel()
    # tests/test_cf90.F90:9-116: nx = 32 non-periodic, omega = 12, f = cos(omega x)
    h = 2 * np.pi / (n - 1)
    x = np.arange(n) * h
    g["cf90_np32_f"] = np.cos(12 * x)
    g["cf90_np32_oracle"] = O.cf90(line3(np.cos(12 * x)), periodic=False).ravel()
    # tests/test_STAGGcd06.F90:1-110: nz = 8 periodic on [0, 1], omega = 1, real and
    # imaginary parts sin / cos(2 pi z) at edges zE and centres zC
    nz = 8
    dz = 1.0 / nz
    zE = np.arange(nz + 1) * dz
    zC = 0.5 * (zE[1:] + zE[:-1])
    w = 2 * np.pi
    for part, fun, dfun, d2fun in (("re", np.sin, np.cos, lambda t: -np.sin(t)),
                                   ("im", np.cos, lambda t: -np.sin(t), lambda t: -np.cos(t))):
        fE, fC = fun(w * zE), fun(w * zC)
        g[f"stagg8_{part}_fE"] = fE
        g[f"stagg8_{part}_fC"] = fC
        g[f"stagg8_{part}_dfC_exact"] = w * dfun(w * zC)
        g[f"stagg8_{part}_dfE_exact"] = w * dfun(w * zE)
        g[f"stagg8_{part}_d2fC_exact"] = w * w * d2fun(w * zC)
        g[f"stagg8_{part}_d2fE_exact"] = w * w * d2fun(w * zE)
        for op, src in (("ddz_E2C", fE), ("ddz_C2E", fC), ("d2dz2_C2C", fC), ("d2dz2_E2E", fE),
                        ("InterpZ_E2C", fE), ("InterpZ_C2E", fC)):
            f3 = np.asfortranarray(src.reshape(1, 1, -1))
            g[f"stagg8_{part}_{op}_oracle"] = O.stagg(f3, nz, dz, op, periodic=True).ravel()
    # seeded lines per family (lines along x; the GPU tests place them along every direction)
    rng = np.random.default_rng(20261203)
    cases = {
        "cd06_p16": (16, lambda f: O.cd06(f, 2 * np.pi / 16, periodic=True)),
        "cd06_np33": (33, lambda f: O.cd06(f, 1.0 / 32, periodic=False)),
        "cd10_p40_d1": (40, lambda f: O.cd10(f, 2 * np.pi / 40, periodic=True, order=1)),
        "cd10_p40_d2": (40, lambda f: O.cd10(f, 2 * np.pi / 40, periodic=True, order=2)),
        "cd10_np27_d1_bc1m1": (27, lambda f: O.cd10(f, 1.0 / 26, periodic=False, bc1=1, bcn=-1, order=1)),
        "cd10_np27_d2_bcm10": (27, lambda f: O.cd10(f, 1.0 / 26, periodic=False, bc1=-1, bcn=0, order=2)),
        "cf90_p24": (24, lambda f: O.cf90(f, periodic=True)),
        "cf90_np24_bc01": (24, lambda f: O.cf90(f, periodic=False, bc1=0, bcn=1)),
        "gaussian_np20": (20, lambda f: O.gaussian(f, periodic=False)),
    }
    for name, (n, fn) in cases.items():
        x = np.arange(n) / n
        f = np.sin(2 * np.pi * 2 * x)[:, None] + 0.3 * rng.standard_normal((n, 3))
        f3 = np.asfortranarray(f.reshape(n, 3, 1))
        g[f"seed_{name}_f"] = f
        g[f"seed_{name}_oracle"] = fn(f3).reshape(n, 3)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **g)
    print(f"wrote {len(g)} arrays to {os.path.join(HERE, 'golden.npz')}")


if __name__ == "__main__":
    main()
