"""The MLP oracle pinned on the CPU: analytic gradient against central finite
differences, Adam against a hand-expanded first step, feature layout."""
import numpy as np

from oracle import mlp


def _random_problem(n=17, seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.2, mlp.N_PARAMS)
    x = rng.normal(0, 1, (n, mlp.N_IN))
    t = rng.normal(0, 1, n)
    return p, x, t


def test_gradient_matches_finite_differences():
    p, x, t = _random_problem()
    _, g = mlp.loss_grad(p, x, t)
    rng = np.random.default_rng(1)
    H, I = mlp.N_HIDDEN, mlp.N_IN
    idx = list(rng.choice(H * I, 40, replace=False))  # W1
    idx += list(H * I + rng.choice(H, 10, replace=False))  # b1
    idx += list(H * I + H + rng.choice(H, 10, replace=False))  # w2
    idx += [mlp.N_PARAMS - 1]  # b2
    fd = mlp.finite_difference_grad(p, x, t, idx)
    assert np.allclose(g[idx], fd, rtol=1e-6, atol=1e-9)


def test_adam_first_step_is_signed_lr():
    # first bias-corrected step: m_hat = g, v_hat = g^2 -> p - lr * g / (|g| + eps)
    g = np.array([0.5, -2.0, 1e-3])
    p, m, v = mlp.adam_step(np.zeros(3), g, np.zeros(3), np.zeros(3), 1, lr=0.01)
    assert np.allclose(p, -0.01 * g / (np.abs(g) + 1e-8))
    assert np.allclose(m, 0.1 * g) and np.allclose(v, 0.001 * g * g)


def test_features_layout():
    f = mlp.features([1.0, 0.1, 1e-3], (3, 1), (2, 1), 1e-8, 7, 1e-4, 1.0)
    assert f.shape == (mlp.N_IN,) and f.dtype == np.float32
    assert np.allclose(f[:3], [0.0, -0.1, -0.3])
    assert np.allclose(f[3:mlp.N_SV], -2.0)  # zero padding at the 1e-20 floor
    assert np.allclose(f[mlp.N_SV:], [0.25, 0.0, -0.8, 0.3, -0.4, 1.0])


def test_predicted_sketch_rounds_up():
    y = np.log2(1 + np.array([0.0, 5.0, 5.2, 100.0]))
    assert list(mlp.predicted_sketch(y)) == [0, 5, 6, 100]
