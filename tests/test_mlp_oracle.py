"""The MLP oracle (oracle/mlp.py) on the CPU: its back-propagated gradient
against central finite differences, its Adam step against the textbook
update, and its default start vector against the library's host function.
No GPU is used."""
import numpy as np

import jupiterncsm_gb300 as jn
from oracle import mlp


def test_backprop_matches_finite_differences():
    rng = np.random.default_rng(3)
    n_in, h, n_out, n = 3, 7, 4, 5
    p = rng.standard_normal(h * n_in + h + h * h + h + n_out * h + n_out) * 0.5
    x, t = rng.standard_normal((n, n_in)), rng.standard_normal((n, n_out))
    _, g = mlp.loss_and_gradient(p, x, t, n_in, h, n_out)
    eps = 1e-6
    fd = np.empty_like(p)
    for i in range(len(p)):
        e = np.zeros_like(p)
        e[i] = eps
        fd[i] = (mlp.loss(p + e, x, t, n_in, h, n_out) - mlp.loss(p - e, x, t, n_in, h, n_out)) / (2 * eps)
    assert np.abs(g - fd).max() < 1e-8 * max(1.0, np.abs(fd).max())


def test_gelu_derivative():
    a = np.linspace(-6, 6, 101)
    fd = (mlp.gelu(a + 1e-6) - mlp.gelu(a - 1e-6)) / 2e-6
    assert np.abs(mlp.gelu_grad(a) - fd).max() < 1e-8


def test_adam_first_step_is_sign_times_lr():
    # with bias correction, the first Adam step moves every parameter by lr * g / (|g| + eps)
    rng = np.random.default_rng(4)
    n_in, h, n_out = 2, 3, 2
    p = rng.standard_normal(h * n_in + h + h * h + h + n_out * h + n_out)
    x, t = rng.standard_normal((4, n_in)), rng.standard_normal((4, n_out))
    _, g = mlp.loss_and_gradient(p, x, t, n_in, h, n_out)
    p1 = mlp.adam(p, x, t, n_in, h, n_out, 1, 0.01)
    assert np.allclose(p - p1, 0.01 * g / (np.abs(g) + 1e-8), rtol=1e-9, atol=1e-15)


def test_default_start_vector_matches_the_library():
    assert np.array_equal(mlp.default_start_vector(1000), jn.default_start_vector(1000))


def test_warm_start_target_ignores_eigenvector_signs():
    rng = np.random.default_rng(5)
    V = np.linalg.qr(rng.standard_normal((50, 6)))[0].T
    r = rng.standard_normal(50)
    flips = np.diag([1, -1, 1, -1, -1, 1.0])
    a, b = mlp.warm_start_targets([V], r)[0], mlp.warm_start_targets([flips @ V], r)[0]
    assert np.allclose(a, b, atol=1e-14)
