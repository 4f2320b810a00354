"""The learned-closure oracle itself (CPU): analytic gradients against finite differences,
the BF16 rounding helper, and the feature definition."""
import numpy as np

from oracle import mlp_oracle as M
from padeops_gb300.sgs_learned import init_params


def test_parameter_count_matches_header():
    from padeops_gb300 import _lib as L

    assert M.NPARAM == L.MLP_NPARAM == 4929


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = init_params(3).astype(np.float64)
    X = rng.standard_normal((37, 10))
    y = 0.02 + 0.01 * rng.random(37)
    loss, g = M.loss_and_grad(p, X, y)
    idx = rng.choice(M.NPARAM, 60, replace=False)
    idx = np.concatenate([idx, [M.NPARAM - 1, 0, 640, 704]])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (M.loss_and_grad(p + e, X, y)[0] - M.loss_and_grad(p - e, X, y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1e-3, abs(g).max()), i


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159, 1e-3], dtype=np.float32)
    b = M.bf16(x)
    assert b[0] == 1.0 and b[1] == 1.0  # ties to even
    assert b[2] == 1.0 + 2 ** -7
    assert abs(b[3] + 3.14159) < 2 ** -7 * 4 and abs(b[4] - 1e-3) < 1e-3 * 2 ** -8


def test_features_are_scale_free_gradients():
    rng = np.random.default_rng(2)
    d = [rng.standard_normal((4, 3, 2)) for _ in range(9)]
    X, mag = M.features(d, 0.5, 1e-3)
    X2, mag2 = M.features([5.0 * a for a in d], 0.5, 1e-3)
    assert np.allclose(X[:, :9], X2[:, :9], rtol=1e-14)
    assert np.allclose(mag2, 5 * mag, rtol=1e-14)
    assert np.allclose(X[:, 9], np.log1p(0.5 * np.sqrt(mag / 1e-3)), rtol=1e-14)
