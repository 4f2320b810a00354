"""Learned closure against the dynamic procedure on the flow statistics (GPU): energy
spectrum per shell, kinetic energy and dissipation after the same number of steps from the
same initial field, next to an untrained network and constant-coefficient Smagorinsky, so
the test shows what training gains over the closure without it."""
import numpy as np
import pytest

import padeops_gb300 as P
from padeops_gb300 import diagnostics as D
from padeops_gb300.sgs_learned import LearnedClosure, init_params, train, training_set
from padeops_gb300.synthetic import hit_initial_field

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N, STEPS = 64, 40


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def _run(u, v, w, steps, closure=None, **kw):
    g = P.igrid()
    g.init(N, N, N, learnedSGS=closure is not None, JudgeFreq=0, **kw)
    if closure is not None:
        g.set_mlp(closure)
    g.set_fields(_dev(u), _dev(v), _dev(w))
    for _ in range(steps):
        g.timeAdvance(use_graph=False)
    return g


def test_spectrum_parseval_and_shells():
    u, v, w = hit_initial_field(N, seed=4)
    g = _run(u, v, w, 0)
    e = D.energy_spectrum(g)
    assert abs(e.sum() - D.kinetic_energy(g)) < 1e-12 * e.sum()
    # the initial field's energy sits in the low shells: E ~ k^4 exp(-2 (k/4)^2) peaks near k = 4
    assert int(np.argmax(e)) in (3, 4, 5)


def test_learned_closure_statistics_against_dynamic():
    # trained on a dynamic run over the same time window, evaluated from another seed
    dyn = _run(*hit_initial_field(N, seed=4), 0)
    trained = LearnedClosure(init_params(0))
    X, y = training_set(dyn, trained, nsteps=STEPS, every=4)
    train(trained, X, y, epochs=10, batch=4096, lr=3e-3)
    u, v, w = hit_initial_field(N, seed=5)
    ref = _run(u, v, w, STEPS)
    e_ref = D.energy_spectrum(ref)
    nu = 1.0 / 1000.0
    eps_ref = D.dissipation(ref, nu)
    out = {}
    for name, g in (("trained", _run(u, v, w, STEPS, trained)),
                    ("trained_planeavg", _run(u, v, w, STEPS, trained, learnedPlaneAvg=True)),
                    ("untrained", _run(u, v, w, STEPS, LearnedClosure(init_params(0)))),
                    ("smagorinsky_0.17", _run(u, v, w, STEPS, DynamicProcedureType=0, Csgs=0.17))):
        c = D.compare_spectra(D.energy_spectrum(g), e_ref, N)
        eps = D.dissipation(g, nu)
        out[name] = (c["max"], c["mean"], abs(eps[1] - eps_ref[1]) / eps_ref[1])
    print({k: tuple(round(x, 4) for x in v) for k, v in out.items()}, "eps_ref", eps_ref)
    # training brings the spectrum and the SGS dissipation closer to the dynamic procedure's
    assert out["trained"][0] < out["untrained"][0]
    assert out["trained"][2] < out["untrained"][2]
    assert out["trained"][0] < 0.05
