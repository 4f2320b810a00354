"""The committed golden fixtures (tests/golden/golden.npz, made by make_golden.py).

CPU: the oracle still reproduces them, and on the reference tests' own inputs it meets the
analytic answers those tests compare against (at the scheme's truncation error).
GPU: the CUDA path reproduces the stored oracle outputs along every direction.
"""
import os

import numpy as np
import pytest

import padeops_gb300 as P
from tests.fields import relerr

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))
EPS = np.finfo(float).eps


def line3(v):
    return np.asfortranarray(np.asarray(v, dtype=np.float64).reshape(-1, 1, 1))


def test_oracle_reproduces_reference_test_cases(oracle):
    n = 256
    h = 2 * np.pi / n
    assert relerr(oracle.cd06(line3(G["cd06_p256_f"]), h).ravel(), G["cd06_p256_oracle"]) <= 4 * EPS
    h = 2 * np.pi / 32
    for d in (1, 2):
        out = oracle.cd10(line3(G["cd10_p32_f"]), h, order=d).ravel()
        assert relerr(out, G[f"cd10_p32_d{d}_oracle"]) <= 4 * EPS
    h = 2 * np.pi / 31
    for d in (1, 2):
        out = oracle.cd10(line3(G["cd10_np32_f"]), h, periodic=False, order=d).ravel()
        assert relerr(out, G[f"cd10_np32_d{d}_oracle"]) <= 4 * EPS
    out = oracle.cf90(line3(G["cf90_np32_f"]), periodic=False).ravel()
    assert relerr(out, G["cf90_np32_oracle"]) <= 4 * EPS


def test_reference_tests_truncation_errors():
    # periodic sin(x) on 256 / 32 points: compact schemes are spectrally close
    assert np.abs(G["cd06_p256_oracle"] - G["cd06_p256_exact"]).max() < 1e-10
    assert np.abs(G["cd10_p32_d1_oracle"] - G["cd10_p32_d1_exact"]).max() < 1e-11
    assert np.abs(G["cd10_p32_d2_oracle"] - G["cd10_p32_d2_exact"]).max() < 1e-10
    # one-sided closures on 32 points (test_cd10_NP.F90): boundary-limited accuracy
    assert np.abs(G["cd10_np32_d1_oracle"] - G["cd10_np32_d1_exact"]).max() < 1e-3
    assert np.abs(G["cd10_np32_d2_oracle"] - G["cd10_np32_d2_exact"]).max() < 1e-2
    # staggered CD06 on 8 points (test_STAGGcd06.F90): sixth order at 8 points per wave
    for p in ("re", "im"):
        assert np.abs(G[f"stagg8_{p}_ddz_E2C_oracle"] - G[f"stagg8_{p}_dfC_exact"]).max() < 1e-3
        assert np.abs(G[f"stagg8_{p}_ddz_C2E_oracle"][:-1] - G[f"stagg8_{p}_dfE_exact"][:-1]).max() < 1e-3
        assert np.abs(G[f"stagg8_{p}_d2dz2_C2C_oracle"] - G[f"stagg8_{p}_d2fC_exact"]).max() < 1e-2


def _seed_cases():
    return sorted({k[5:-2] for k in G.files if k.startswith("seed_") and k.endswith("_f")})


@pytest.mark.parametrize("case", _seed_cases())
def test_oracle_reproduces_seeded_lines(oracle, case):
    f = G[f"seed_{case}_f"]
    n = f.shape[0]
    f3 = np.asfortranarray(f.reshape(n, 3, 1))
    fam = case.split("_")[0]
    if fam == "cd06":
        per = case.startswith("cd06_p")
        out = oracle.cd06(f3, 2 * np.pi / n if per else 1.0 / (n - 1), periodic=per)
    elif fam == "cd10":
        per = "_p" in case
        order = 2 if "_d2" in case else 1
        bc = {"bc1m1": (1, -1), "bcm10": (-1, 0)}.get(case.split("_")[-1], (0, 0))
        out = oracle.cd10(f3, 2 * np.pi / n if per else 1.0 / (n - 1), periodic=per, bc1=bc[0], bcn=bc[1],
                          order=order)
    elif fam == "cf90":
        per = "_p" in case
        bc = (0, 1) if case.endswith("bc01") else (0, 0)
        out = oracle.cf90(f3, periodic=per, bc1=bc[0], bcn=bc[1])
    else:
        out = oracle.gaussian(f3, periodic=False)
    assert relerr(out.reshape(n, 3), G[f"seed_{case}_oracle"]) <= 8 * EPS


# ---------------------------------------------------------------- GPU


def _gpu_apply(obj, opcode, f_line, dir, bc=(0, 0), cplx_im=None):
    """Place the line(s) along `dir` of a small 3-D array (other extents 3 x 2), run, return lines."""
    import torch

    fl = np.atleast_2d(np.asarray(f_line).T).T  # (n, k)
    n, k = fl.shape
    shape = [k, 2]
    shape.insert(dir - 1, n)
    f3 = np.zeros(shape)
    idx = [slice(None)] * 3
    for j in range(k):
        for b in range(2):
            sl = [j, b]
            sl.insert(dir - 1, slice(None))
            f3[tuple(sl)] = fl[:, j]
    f3 = np.asfortranarray(f3)
    dev = torch.from_numpy(np.ascontiguousarray(f3.T)).cuda()
    n_out = obj.lengths(opcode)[1]
    oshape = list(shape)
    oshape[dir - 1] = n_out
    out = torch.empty(tuple(reversed(oshape)), dtype=torch.float64, device="cuda")
    obj.apply(opcode, dir, dev, out, k, 2, *bc)
    torch.cuda.synchronize()
    o3 = np.asfortranarray(out.cpu().numpy().T)
    res = np.zeros((n_out, k))
    for j in range(k):
        sl = [j, 1]
        sl.insert(dir - 1, slice(None))
        res[:, j] = o3[tuple(sl)]
    del idx
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("dir", [1, 2, 3])
def test_cuda_path_matches_golden(dir):
    pytest.importorskip("torch")
    o = P.cd10()
    assert o.init(32, 2 * np.pi / 32, True) == 0
    for d in (1, 2):
        out = _gpu_apply(o, d, G["cd10_p32_f"], dir).ravel()
        assert relerr(out, G[f"cd10_p32_d{d}_oracle"]) < 1e-12
    o = P.cd10()
    assert o.init(32, 2 * np.pi / 31, False) == 0
    for d in (1, 2):
        out = _gpu_apply(o, d, G["cd10_np32_f"], dir).ravel()
        # one-sided second-derivative closures amplify the double-float 2^-48 representation
        # error by their coefficient sums (~1e3): 1e-10 for d2, as for the seeded d2 lines
        assert relerr(out, G[f"cd10_np32_d{d}_oracle"]) < (1e-12 if d == 1 else 1e-10)
    c = P.cd06()
    assert c.init(256, 2 * np.pi / 256, True) == 0
    assert relerr(_gpu_apply(c, 1, G["cd06_p256_f"], dir).ravel(), G["cd06_p256_oracle"]) < 1e-12
    f = P.cf90()
    assert f.init(32, False) == 0
    assert relerr(_gpu_apply(f, 0, G["cf90_np32_f"], dir).ravel(), G["cf90_np32_oracle"]) < 1e-12
    for case in _seed_cases():
        fl = G[f"seed_{case}_f"]
        n = fl.shape[0]
        fam = case.split("_")[0]
        bc = (0, 0)
        if fam == "cd06":
            per = case.startswith("cd06_p")
            obj, opc = P.cd06(), 1
            assert obj.init(n, 2 * np.pi / n if per else 1.0 / (n - 1), per) == 0
        elif fam == "cd10":
            per = "_p" in case
            obj, opc = P.cd10(), (2 if "_d2" in case else 1)
            assert obj.init(n, 2 * np.pi / n if per else 1.0 / (n - 1), per) == 0
            bc = {"bc1m1": (1, -1), "bcm10": (-1, 0)}.get(case.split("_")[-1], (0, 0))
        elif fam == "cf90":
            per = "_p" in case
            obj, opc = P.cf90(), 0
            assert obj.init(n, per) == 0
            bc = (0, 1) if case.endswith("bc01") else (0, 0)
        else:
            obj, opc = P.gaussian(), 0
            assert obj.init(n, False) == 0
        out = _gpu_apply(obj, opc, fl, dir, bc)
        tol = 1e-10 if "_d2" in case else 1e-12
        assert relerr(out, G[f"seed_{case}_oracle"]) < tol, case


@pytest.mark.gpu
def test_cuda_stagg_matches_golden():
    pytest.importorskip("torch")
    st = P.cd06stagg()
    nz = 8
    assert st.init(nz, 1.0 / nz) == 0
    ops = ["ddz_E2C", "ddz_C2E", "d2dz2_C2C", "d2dz2_E2E", "InterpZ_E2C", "InterpZ_C2E"]
    from padeops_gb300 import _lib as L

    for p in ("re", "im"):
        for op in ops:
            src = G[f"stagg8_{p}_fE"] if op in ("ddz_E2C", "d2dz2_E2E", "InterpZ_E2C") else G[f"stagg8_{p}_fC"]
            out = _gpu_apply(st, L.STAGG_OPS.index(op), src, 3).ravel()
            tol = 1e-10 if op.startswith("d2") else 1e-12
            assert relerr(out, G[f"stagg8_{p}_{op}_oracle"]) < tol, (p, op)
