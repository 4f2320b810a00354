"""The learned closure's fallback and judge inside the LES step (GPU).

* Points whose features leave the closure's training range take the fallback coefficient:
  before any judge step that is the constant Smagorinsky (Csgs Delta)^2, so with a range no
  point fits, the learned run's eddy viscosity is the constant-coefficient model's (to the
  FP32 |S| the inference kernel works with: 1e-6 relative).
* Every JudgeFreq steps the dynamic procedure judges the closure: the reported error is the
  relative difference of the closure's plane-averaged Cs^2 Delta^2 and lambda(z); above
  JudgeTol every later stage takes lambda(z) |S| (counted per point evaluation).
* The direct-simulation training set (dns_training_set) on a small grid.
"""
import numpy as np
import pytest

import padeops_gb300 as P
from padeops_gb300.sgs_learned import LearnedClosure, box_filter, delta_les, dns_training_set, init_params, train
from padeops_gb300.synthetic import hit_initial_field
from tests.fields import relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()


def host(t):
    return np.asfortranarray(t.cpu().numpy().T)


def _grid(n, **kw):
    u, v, w = hit_initial_field(n, seed=4)
    g = P.igrid()
    g.init(n, n, n, **kw)
    g.set_fields(dev(u), dev(v), dev(w))
    return g


def test_out_of_range_points_take_the_constant_coefficient():
    n = 16
    clo = LearnedClosure(init_params(3))
    clo.set_range(np.full(10, 50.0), np.full(10, 60.0))  # no feature vector fits
    a = _grid(n, learnedSGS=True, JudgeFreq=0)
    a.set_mlp(clo)
    b = _grid(n, DynamicProcedureType=0)  # constant Smagorinsky, Csgs 0.17
    a.timeAdvance(use_graph=False)
    b.timeAdvance(use_graph=False)
    assert relerr(host(a.field("nu_sgs_C")), host(b.field("nu_sgs_C"))) < 1e-6
    assert a.judge_info()["n_fallback"] == 3 * n ** 3  # every point of every stage
    # without a range the network's own coefficient is used
    clo.set_range(None, None)
    c = _grid(n, learnedSGS=True, JudgeFreq=0)
    c.set_mlp(clo)
    c.timeAdvance(use_graph=False)
    assert c.judge_info()["n_fallback"] == 0
    assert relerr(host(c.field("nu_sgs_C")), host(b.field("nu_sgs_C"))) > 1e-3


def test_judge_error_and_switch_to_the_dynamic_coefficient():
    n = 16
    clo = LearnedClosure(init_params(3))
    g = _grid(n, learnedSGS=True, JudgeFreq=1, JudgeTol=1e-12)
    g.set_mlp(clo)
    assert g.judge_info()["err"] == -1.0  # no judge step yet
    g.timeAdvance(use_graph=False)
    j = g.judge_info()
    lam = g.info()["lambda"]
    lc = j["lambda_closure"]
    assert np.isfinite(lc).all() and lc.min() >= 0
    scale = max(np.abs(lam).max(), np.abs(lc).max())
    assert j["err"] == pytest.approx(np.abs(lc - lam).max() / scale, rel=1e-12)
    assert 0.0 <= j["err"] <= 1.0
    assert j["err"] > 1e-12
    # the switch is on after stage 1: stages 2 and 3 took lambda(z) |S| at every point
    assert j["n_fallback"] == 2 * n ** 3
    # a generous tolerance keeps the closure
    h = _grid(n, learnedSGS=True, JudgeFreq=1, JudgeTol=1e9)
    h.set_mlp(clo)
    h.timeAdvance(use_graph=False)
    assert h.judge_info()["n_fallback"] == 0


def test_box_filter_is_a_block_mean():
    rng = np.random.default_rng(2)
    f = torch.from_numpy(rng.standard_normal((8, 12, 16)))
    got = box_filter(f, 4).numpy()
    ref = f.numpy().reshape(2, 4, 3, 4, 4, 4).mean(axis=(1, 3, 5))
    assert np.allclose(got, ref, rtol=0, atol=1e-15)


def test_dns_training_set_and_training():
    X, y, info = dns_training_set(n_dns=64, ratio=4, nsteps=4, snapshots=2, every=2, seed=5, kp=8.0)
    assert X.shape == (2 * 16 ** 3, 10) and y.shape == (2 * 16 ** 3,)
    assert torch.isfinite(X).all() and torch.isfinite(y).all()
    assert float(y.min()) >= 0.0 and float(y.max()) <= 0.25 and float(y.mean()) > 0.0
    assert info["n_les"] == 16 and info["samples"] == X.shape[0]
    clo = LearnedClosure(init_params(0))
    hist = train(clo, X, y, epochs=3, batch=512, lr=3e-3)
    assert hist[-1] < hist[0]
    # the training range was recorded: points of this set are inside it
    dl = delta_les(2 * np.pi / 16, 2 * np.pi / 16, 2 * np.pi / 16)
    assert dl > 0
