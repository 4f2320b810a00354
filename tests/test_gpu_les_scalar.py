"""The scalar SGS flux divergence (getRHS_SGS_Scalar / getQjSGS, sgsmod_igrid.F90:268-335;
DoStandardDynamicProcedureScalar, standardDynamicProcedure.F90:1-71) against the oracle's
restatement on the GPU LES's own state (GPU).

Tolerances: 1e-10 normwise for the updated right-hand side (the same FFT / compact-solve
chains as the LES step), 1e-9 for the planar ratio Beta(z), as for the momentum procedure's
lambda(z) in tests/test_gpu_les.py."""
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


def _smooth(rng, shape, kmax=4):
    x = [np.arange(s) * 2 * np.pi / s for s in shape]
    f = np.zeros(shape)
    for _ in range(6):
        k = rng.integers(-kmax, kmax + 1, 3)
        ph = rng.uniform(0, 2 * np.pi)
        f += rng.standard_normal() * np.cos(k[0] * x[0][:, None, None] + k[1] * x[1][None, :, None]
                                            + k[2] * x[2][None, None, :] + ph)
    return np.asfortranarray(f)


@pytest.mark.parametrize("dynamic", [False, True], ids=["nu_over_Pr", "dynamic"])
def test_scalar_sgs_matches_oracle(dynamic):
    n, L_ = 16, 2 * np.pi
    u, v, w = hit_initial_field(n, seed=6)
    g = P.igrid()
    g.init(n, n, n, DynamicProcedureType=1)
    g.set_fields(dev(u), dev(v), dev(w))
    g.timeAdvance(use_graph=False)
    ref = LesOracle(n, n, n, L_, L_, L_)
    fields = {name: host(g.field(name)) for name in ("u", "v", "wC", "uhat", "vhat", "what")}
    fields["whatC"] = ref.sz(fields["what"], "InterpZ_E2C")
    fields["duidxjC"] = [host(g.field(f"duidxjC{i + 1}")) for i in range(9)]
    fields["nuC"], fields["nuE"] = host(g.field("nu_sgs_C")), host(g.field("nu_sgs_E"))
    rng = np.random.default_rng(3)
    T = _smooth(rng, (n, n, n))
    That = ref.fft(T)
    dT = [_smooth(rng, (n, n, n)) for _ in range(3)]
    dTdzE = _smooth(rng, (n, n, n + 1))
    Trhs0 = ref.fft(_smooth(rng, (n, n, n)))
    Trhs = dev(Trhs0)
    beta = g.scalar_sgs(dev(T), dev(That), dev(dT[0]), dev(dT[1]), dev(dT[2]), dev(dTdzE), Trhs, Pr=0.7,
                        dynamic=dynamic)
    torch.cuda.synchronize()
    want, rbeta = ref.scalar_sgs_rhs(T, That, dT, dTdzE, Trhs0, Pr=0.7, dynamic=dynamic, fields=fields)
    got = host(Trhs)
    assert relerr(got - Trhs0, want - Trhs0) < 1e-10  # the SGS part itself
    if dynamic:
        assert np.all(rbeta >= 0) and rbeta.max() > 0
        assert relerr(beta, rbeta) < 1e-9
