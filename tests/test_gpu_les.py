"""The periodic LES step (igrid TVD-RK3 + dynamic Smagorinsky) against the oracle (GPU).

Tolerances (normwise relative): fields after the init sequence 1e-12; after one and two
time steps 1e-10 (each stage chains ~40 FFTs and ~20 compact solves whose FP64 results
differ from numpy's/the oracle's in the last bits; the step then amplifies them by the
advection and the SGS model's |S| nonlinearity).  The dynamic coefficient is a ratio of
planar averages: 1e-9.
"""
import numpy as np
import pytest

import padeops_gb300 as P
from oracle.les_oracle import LesOracle
from padeops_gb300.synthetic import hit_initial_field
from tests.fields import relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()


def host(t):
    return np.asfortranarray(t.cpu().numpy().T)


def _pair(n, oracle, **kw):
    L_ = 2 * np.pi
    u, v, w = hit_initial_field(n, seed=4)
    ref = LesOracle(n, n, n, L_, L_, L_, **kw)
    ref.init_fields(u, v, w)
    g = P.igrid()
    okw = dict(kw)
    if "dynamic" in okw:
        okw["DynamicProcedureType"] = 1 if okw.pop("dynamic") else 0
    g.init(n, n, n, **okw)
    g.set_fields(dev(u), dev(v), dev(w))
    return g, ref


FIELDS = ["u", "v", "wC", "w", "uE", "vE"]


def _compare(g, ref, tol):
    for name in FIELDS:
        assert relerr(host(g.field(name)), getattr(ref, name)) < tol, name
    for i in range(9):
        assert relerr(host(g.field(f"duidxjC{i + 1}")), ref.duidxjC[i]) < tol, ("duidxjC", i + 1)
        assert relerr(host(g.field(f"duidxjE{i + 1}")), ref.duidxjE[i]) < tol, ("duidxjE", i + 1)
    for name, arr in (("uhat", ref.uhat), ("vhat", ref.vhat), ("what", ref.what)):
        assert relerr(host(g.field(name)), arr) < tol, name


def test_init_sequence_matches_oracle(oracle):
    g, ref = _pair(16, oracle)
    _compare(g, ref, 1e-12)


def test_init_sequence_with_disparate_magnitudes(oracle):
    """Velocity components 1e6 apart: transforms that share a launch keep each field's own
    scaling, so the small component's gradients stay at full relative precision."""
    n, L_ = 16, 2 * np.pi
    u, v, w = hit_initial_field(n, seed=4)
    v = 1e-6 * v
    w = 1e3 * w
    ref = LesOracle(n, n, n, L_, L_, L_)
    ref.init_fields(u, v, w)
    g = P.igrid()
    g.init(n, n, n)
    g.set_fields(dev(u), dev(v), dev(w))
    _compare(g, ref, 1e-12)
    g.timeAdvance(use_graph=False)  # the right-hand sides pair transforms of u and v too
    ref.tvd_rk3()
    _compare(g, ref, 1e-10)


@pytest.mark.parametrize("kw", [dict(dynamic=True), dict(dynamic=False), dict(useSGS=False),
                                dict(useSGS=False, isInviscid=True), dict(dynamic=False, SGSModelID=1),
                                dict(dynamic=False, SGSModelID=2)])
def test_two_steps_match_oracle(oracle, kw):
    g, ref = _pair(16, oracle, **kw)
    for step in range(2):
        g.timeAdvance(use_graph=False)
        dt = ref.tvd_rk3()
        info = g.info()
        assert info["step"] == step + 1
        assert info["dt"] == pytest.approx(dt, rel=1e-12)
        assert info["tsim"] == pytest.approx(ref.tsim, rel=1e-12)
        _compare(g, ref, 1e-10)
        if kw.get("dynamic", True) and kw.get("useSGS", True):
            lam = info["lambda"]
            assert np.max(np.abs(lam - ref.lambda1d)) <= 1e-9 * np.max(np.abs(ref.lambda1d))
            assert float(g.field("nu_sgs_C").min()) >= 0.0


def test_two_steps_native_fp64_transforms(oracle, native_lib):
    """The same step with the FP64 transform kernels, which take the fields and their x
    gradients from separate y transforms (the double-float path shares one)."""
    from padeops_gb300 import _lib as L

    old = native_lib.pade_fft_get_arith()
    L.check(native_lib.pade_fft_set_arith(L.FFT_FP64))
    try:
        g, ref = _pair(16, oracle)
        _compare(g, ref, 1e-12)
        for _ in range(2):
            g.timeAdvance(use_graph=False)
            ref.tvd_rk3()
            _compare(g, ref, 1e-10)
    finally:
        native_lib.pade_fft_set_arith(old)


def test_graph_replay_equals_eager(oracle):
    ga, _ = _pair(16, oracle)
    gb, _ = _pair(16, oracle)
    side = torch.cuda.Stream()  # graphs are captured on a non-default stream
    for _ in range(3):  # step 0 runs eagerly (divergence check), steps 1-2 replay the graph
        ga.timeAdvance(use_graph=False)
        with torch.cuda.stream(side):
            gb.timeAdvance(use_graph=True)
        side.synchronize()
    torch.cuda.synchronize()
    for name in ("uhat", "vhat", "what", "u", "wC"):
        assert torch.equal(ga.field(name), gb.field(name)), name
    assert ga.info()["tsim"] == gb.info()["tsim"]


def test_larger_grid_and_divergence(oracle):
    n = 32
    g, ref = _pair(n, oracle)
    g.timeAdvance(use_graph=False)
    ref.tvd_rk3()
    _compare(g, ref, 1e-10)
    # the projected velocity is discretely divergence free
    sp = P.spectral()
    d = 2 * np.pi / n
    sp.init(n, n, n, d, d, fixOddball=False)
    po = P.padepoisson()
    po.init(d, d, d, sp)
    div = torch.empty((n, n, n), dtype=torch.float64, device="cuda")
    U, V, W = g.field("uhat").clone(), g.field("vhat").clone(), g.field("what").clone()
    po.DivergenceCheck(U, V, W, div)
    assert float(div.abs().max()) < 1e-12 * float(g.field("u").abs().max()) * n
