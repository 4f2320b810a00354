"""Properties of the LES oracle (CPU): the reference's conservation and model identities."""
import numpy as np
import pytest

from oracle.les_oracle import LesOracle
from padeops_gb300.synthetic import hit_initial_field


@pytest.fixture(scope="module")
def built(oracle):
    return oracle


def _les(n=16, **kw):
    u, v, w = hit_initial_field(n, seed=4)
    L_ = 2 * np.pi
    les = LesOracle(n, n, n, L_, L_, L_, **kw)
    les.init_fields(u, v, w)
    return les


def _ke(les):
    return 0.5 * np.mean(les.u ** 2 + les.v ** 2 + les.wC ** 2)


def test_initial_field_is_projected_and_normalised(built):
    u, v, w = hit_initial_field(16, seed=4)
    assert np.sqrt((u ** 2 + v ** 2 + w[:, :, :-1] ** 2).mean() / 3) == pytest.approx(1.0, rel=1e-12)
    les = _les()
    assert np.abs(les.divergence(les.uhat, les.vhat, les.what)).max() < 1e-13
    # the projection removes the compressive third of an isotropic random field's energy
    assert 0.8 < _ke(les) < 1.2


def test_edge_planes_are_periodic(built):
    les = _les()
    assert np.array_equal(les.what[:, :, -1], les.what[:, :, 0])
    assert np.abs(les.w[:, :, -1] - les.w[:, :, 0]).max() < 1e-13


def test_energy_decays_with_viscosity_and_sgs(built):
    les = _les()
    e0 = _ke(les)
    for _ in range(3):
        les.tvd_rk3()
    assert _ke(les) < e0
    assert np.abs(les.divergence(les.uhat, les.vhat, les.what)).max() < 1e-12


def test_inviscid_energy_nearly_conserved(built):
    les = _les(useSGS=False, isInviscid=True)
    e0 = _ke(les)
    les.tvd_rk3(dt=1e-3)
    assert abs(_ke(les) - e0) < 1e-4 * e0


def test_cfl_time_step(built):
    les = _les(CFL=0.5, Re=1e8)
    dt = les.compute_deltaT()
    ts = np.abs(les.u / les.dx) + np.abs(les.v / les.dy) + np.abs(les.wC / les.dz)
    assert dt == pytest.approx(0.5 / ts.max(), rel=1e-14)
    les2 = _les(CFL=0.5, Re=1e-3)  # viscous limit CFL*Re*min(d)^2
    assert les2.compute_deltaT() == pytest.approx(0.5 * 1e-3 * les2.dx ** 2, rel=1e-14)


def test_smagorinsky_kernel_is_sqrt_2SijSij(built):
    rng = np.random.default_rng(0)
    d = [rng.standard_normal((4, 3, 2)) for _ in range(9)]
    S = LesOracle.sij(d)
    full = np.zeros((4, 3, 2))
    G = np.array(d).reshape(3, 3, 4, 3, 2)
    for i in range(3):
        for j in range(3):
            sij = 0.5 * (G[i, j] + G[j, i])
            full += sij * sij
    assert np.allclose(LesOracle.smag_kernel(S), np.sqrt(2 * full), rtol=1e-14)


def test_dynamic_coefficient_nonnegative_and_planar(built):
    les = _les()
    les.tvd_rk3()
    assert les.lambda1d.shape == (16,)
    assert np.all(les.lambda1d >= 0)
    assert les.lambda1d.max() > 0


def _grad_list(g):
    """(3, 3, ...) gradient g[i, j] = d u_i / d x_j -> the 9-array list duidxj(1..9)."""
    return [g[i, j] for i in range(3) for j in range(3)]


def test_sigma_kernel_against_singular_values():
    """sigma.F90: nu / (C Delta)^2 = s3 (s1 - s2)(s2 - s3) / s1^2 from the singular values
    of the velocity gradient: zero for pure shear, solid rotation and axisymmetric strain
    (the model's defining properties), and the SVD value for general gradients."""
    from oracle.les_oracle import LesOracle as LO

    special = [np.array([[0, 1, 0], [0, 0, 0], [0, 0, 0]], float),
               np.array([[0, 1, 0], [-1, 0, 0], [0, 0, 0]], float),
               np.diag([1.0, -0.5, -0.5])]
    for g in special:
        nu = LO.sigma_kernel(_grad_list(g[:, :, None]))
        # acos at exactly +-1 (equal singular values) turns the reference's 1e-13
        # regularisation and last-bit rounding into ~sqrt(eps) of the gradient scale
        assert abs(float(nu[0])) < 1e-6
    rng = np.random.default_rng(3)
    G = rng.standard_normal((3, 3, 200))
    nu = LO.sigma_kernel(_grad_list(G))
    s = np.linalg.svd(np.moveaxis(G, 2, 0), compute_uv=False)  # descending
    ref = s[:, 2] * (s[:, 0] - s[:, 1]) * (s[:, 1] - s[:, 2]) / (s[:, 0] ** 2)
    assert np.max(np.abs(nu - ref)) < 1e-9 * np.max(np.abs(ref))
    assert np.all(nu >= 0)


def test_amd_kernel_against_contraction():
    """AMD.F90: nu = max(-(C_k g_ik)(C_k g_jk) S_ij / (g_lm g_lm), 0)."""
    from oracle.les_oracle import LesOracle as LO

    rng = np.random.default_rng(4)
    G = rng.standard_normal((3, 3, 100))
    c = (0.3, 0.2, 0.1)
    S = 0.5 * (G + np.swapaxes(G, 0, 1))
    Gs = G * np.array(c)[None, :, None]
    num = np.einsum("ikn,jkn,ijn->n", Gs, Gs, S)
    ref = np.maximum(-num / np.einsum("ijn,ijn->n", G, G), 0.0)
    Sl = [S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2], S[2, 2]]
    nu = LO.amd_kernel(_grad_list(G), Sl, c)
    assert np.max(np.abs(nu - ref)) < 1e-14 * np.max(np.abs(ref))
    assert np.count_nonzero(nu) > 10 and np.count_nonzero(nu == 0) > 10  # both signs of num occur


def test_scalar_sgs_restatement_known_answer():
    """With a constant kappa = nu / Pr, the flux divergence of -kappa grad T adds kappa
    d2T/dx2 to the scalar's right-hand side (a single x mode here)."""
    from oracle.les_oracle import LesOracle

    n, L_ = 16, 2 * np.pi
    o = LesOracle(n, n, n, L_, L_, L_)
    x = (np.arange(n) * L_ / n)[:, None, None] * np.ones((1, n, n))
    T = np.asfortranarray(np.cos(2 * x))
    dT = [-2 * np.sin(2 * x), np.zeros_like(x), np.zeros_like(x)]
    nu = 0.3
    fields = {"nuC": np.full((n, n, n), nu), "nuE": np.full((n, n, n + 1), nu)}
    Trhs0 = np.zeros((n // 2 + 1, n, n), dtype=complex)
    Trhs, beta = o.scalar_sgs_rhs(T, o.fft(T), dT, np.zeros((n, n, n + 1)), Trhs0, Pr=0.6, fields=fields)
    assert beta is None
    want = o.fft((nu / 0.6) * (-4.0) * np.cos(2 * x))
    assert np.abs(Trhs - want).max() <= 1e-12 * np.abs(want).max()
