"""The learned SGS closure's kernels against the FP64 oracle, and the LES step using it (GPU).

Tolerances: FP32 training kernels vs FP64 oracle 1e-4 (loss, gradient) and 1e-5 (AdamW
parameters); features 1e-6; BF16 tensor-core inference 5e-3 of nu (BF16 carries 8 bits
of mantissa; the oracle rounds operands and activations the same way but sums in a
different order and evaluates GELU exactly, where the kernel uses BF16 arithmetic and an
approximate tanh: about 1e-3 on these networks).
"""
import numpy as np
import pytest

import padeops_gb300 as P
from padeops_gb300 import _lib as L
from oracle import mlp_oracle as M
from padeops_gb300.synthetic import hit_initial_field
from padeops_gb300.sgs_learned import LearnedClosure, delta_les, init_params, train, training_set
from tests.fields import relerr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _data(B, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((B, 10)).astype(np.float32)
    y = (0.02 + 0.02 * rng.random(B)).astype(np.float32)
    return X, y


@pytest.mark.parametrize("B", [1, 128, 300, 4096])
def test_loss_and_gradient_match_oracle(B):
    p = init_params(5)
    X, y = _data(B, B)
    c = LearnedClosure(p)
    loss, g = c.loss_grad(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda())
    rl, rg = M.loss_and_grad(p.astype(np.float64), X.astype(np.float64), y.astype(np.float64))
    assert abs(loss - rl) <= 1e-4 * abs(rl)
    assert relerr(g, rg) < 1e-4


def test_adamw_steps_match_oracle():
    p = init_params(6)
    X, y = _data(512, 7)
    c = LearnedClosure(p)
    Xd, yd = torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda()
    q = p.astype(np.float64)
    m = np.zeros_like(q)
    v = np.zeros_like(q)
    for t in range(1, 4):
        c.train_step(Xd, yd, lr=1e-3, wd=1e-2)
        _, g = M.loss_and_grad(q, X.astype(np.float64), y.astype(np.float64))
        q, m, v = M.adamw(q, g, m, v, t, 1e-3, 1e-2)
    assert relerr(c.get_params(), q) < 1e-5


def _grads(shape, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(shape) for _ in range(9)]


def test_features_and_inference_match_oracle():
    shape = (40, 24, 9)  # 8640 points: tiles of 128 with a ragged end
    d = _grads(shape, 3)
    dd = [torch.from_numpy(np.ascontiguousarray(a.T)).cuda() for a in d]
    delta, nu = 0.3, 1e-3
    p = init_params(8)
    c = LearnedClosure(p)
    X = c.features(dd, delta, nu).cpu().numpy()
    rX, mag = M.features(d, delta, nu)
    assert relerr(X, rX) < 1e-6
    out, cs2 = c.infer_nu(dd, delta, nu, want_cs2=True)
    import ctypes

    flag = ctypes.c_int(-1)
    assert L.lib().pade_mlp_status(ctypes.byref(flag)) == 0 and flag.value == 0  # no tensor-core wait gave up
    rcs2 = M.infer_bf16(p.astype(np.float64), rX.astype(np.float32).astype(np.float64))
    assert relerr(cs2.cpu().numpy(), rcs2) < 5e-3
    assert relerr(out.cpu().numpy(), rcs2 * delta ** 2 * mag) < 5e-3
    # the exact-FP64 model is within BF16 accuracy too
    full, _ = M.forward(p.astype(np.float64), rX)
    assert relerr(cs2.cpu().numpy(), full) < 2e-2


def test_learned_les_trains_and_runs():
    n = 32
    L_ = 2 * np.pi
    u, v, w = hit_initial_field(n, seed=4)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # noqa: E731
    dyn = P.igrid()
    dyn.init(n, n, n)
    dyn.set_fields(dev(u), dev(v), dev(w))
    c = LearnedClosure(init_params(0))
    X, y = training_set(dyn, c, nsteps=4, every=1)
    hist = train(c, X, y, epochs=8, batch=2048, lr=3e-3)
    assert hist[-1] < hist[0]
    ref = P.igrid()
    ref.init(n, n, n)
    ref.set_fields(dev(u), dev(v), dev(w))
    lg = P.igrid()
    lg.init(n, n, n, learnedSGS=True, JudgeFreq=2)
    lg.set_mlp(c)
    lg.set_fields(dev(u), dev(v), dev(w))
    for _ in range(4):
        ref.timeAdvance(use_graph=False)
        lg.timeAdvance(use_graph=False)
    ke = lambda g: float(0.5 * (g.field("u") ** 2 + g.field("v") ** 2 + g.field("wC") ** 2).mean())  # noqa: E731
    assert np.isfinite(ke(lg))
    assert abs(ke(lg) - ke(ref)) < 0.02 * ke(ref)
    nuC = lg.field("nu_sgs_C")
    assert float(nuC.min()) >= 0.0
    # the learned coefficient follows the dynamic one it was trained on
    dl = delta_les(L_ / n, L_ / n, L_ / n)
    lam = lg.info()["lambda"]  # the judge's dynamic coefficient
    grads = [lg.field(f"duidxjC{i + 1}") for i in range(9)]
    _, cs2 = c.infer_nu(grads, dl, 1.0 / 1000.0, want_cs2=True)
    assert abs(float(cs2.mean()) - lam.mean() / dl ** 2) < 0.5 * lam.mean() / dl ** 2
    # graph replay with the closure (no judge) equals eager stepping
    ga, gb = P.igrid(), P.igrid()
    for g in (ga, gb):
        g.init(16, 16, 16, learnedSGS=True, JudgeFreq=0)
        g.set_mlp(c)
        u2, v2, w2 = hit_initial_field(16, seed=4)
        g.set_fields(dev(u2), dev(v2), dev(w2))
    side = torch.cuda.Stream()
    for _ in range(3):
        ga.timeAdvance(use_graph=False)
        with torch.cuda.stream(side):
            gb.timeAdvance(use_graph=True)
        side.synchronize()
    assert torch.equal(ga.field("uhat"), gb.field("uhat"))
