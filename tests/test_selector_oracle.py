"""CPU checks of the selector oracle: the analytic MLP gradient against
central differences, and the feature restatement on matrices whose answers are
known in closed form."""
import numpy as np

from oracle import selector_ref as sr


def _params(seed):
    rng = np.random.default_rng(seed)
    p = rng.standard_normal(sr.NPARAM + 32) * 0.3
    p[sr.NPARAM:sr.NPARAM + 16] = rng.standard_normal(16)          # means
    p[sr.NPARAM + 16:] = 0.5 + rng.random(16)                      # std devs
    return p


def test_mlp_analytic_gradient_matches_central_differences():
    rng = np.random.default_rng(1)
    p = _params(2)
    X = rng.standard_normal((40, 16))
    y = rng.integers(0, 3, size=40)
    loss, g = sr.mlp_loss_grad(p, X, y)
    assert g.shape == (sr.NPARAM,) and np.isfinite(loss)
    idx = np.concatenate([rng.choice(sr.NPARAM, 60, replace=False),
                          np.arange(sr.NPARAM - 3, sr.NPARAM)])
    num = sr.numeric_grad(p, X, y, idx)
    assert np.allclose(g[idx], num, rtol=1e-5, atol=1e-8)


def test_mlp_expected_cost_gradient_matches_central_differences():
    rng = np.random.default_rng(11)
    p = _params(12)
    X = rng.standard_normal((40, 16))
    cost = rng.random((40, 3)) * 3.0
    loss, g = sr.mlp_cost_grad(p, X, cost)
    assert g.shape == (sr.NPARAM,) and np.isfinite(loss)
    idx = np.concatenate([rng.choice(sr.NPARAM, 60, replace=False),
                          np.arange(sr.NPARAM - 3, sr.NPARAM)])
    num = sr.numeric_grad(p, X, cost, idx, loss_fn=sr.mlp_cost_grad)
    assert np.allclose(g[idx], num, rtol=1e-5, atol=1e-8)
    # a cost vector that is the same for every class has no gradient
    flat = np.repeat(cost[:, :1], 3, axis=1)
    assert np.allclose(sr.mlp_cost_grad(p, X, flat)[1], 0.0, atol=1e-12)


def test_mlp_forward_is_a_distribution():
    rng = np.random.default_rng(3)
    pr = sr.mlp_forward(_params(4), rng.standard_normal((25, 16)))
    assert pr.shape == (25, 3)
    assert np.allclose(pr.sum(1), 1.0) and (pr >= 0).all()


def test_features_of_diagonal_matrix():
    d = np.array([4.0, 2.0, 1.0, 0.25])
    f = sr.features(np.diag(d), 2)
    assert np.isclose(f[0], np.log2(4) / 9) and np.isclose(f[1], 0.5)
    assert np.isclose(f[2], np.log10(4.0)) and np.isclose(f[5], np.log10(4.0))
    assert np.isclose(f[6], np.log10(4.0), atol=1e-9)          # sigma_max exactly
    assert np.isclose(f[15], np.log10(16.0), atol=1e-9)        # kappa_2 exactly (n <= 4 steps)
    assert f[10] == 1.0 and f[13] == 0.0


def test_features_kappa_estimate_bounds_true_kappa():
    rng = np.random.default_rng(5)
    for n, lk in [(40, 3.0), (120, 8.0)]:
        u, _ = np.linalg.qr(rng.standard_normal((n, n)))
        v, _ = np.linalg.qr(rng.standard_normal((n, n)))
        s = 10.0 ** (-lk * np.arange(n) / (n - 1))
        a = (u * s) @ v.T
        f = sr.features(a, 1)
        assert np.isclose(f[6], 0.0, atol=0.05)                # sigma_max = 1
        assert 0.0 < f[15] <= lk + 1e-6                         # Ritz bound <= log10 kappa
