"""The learned warm start on the GPU: the MLP kernels against the float64
oracle (oracle/mlp.py), and what the trained network gains over the batched
solver's default start.

Tolerances: the kernels compute in FP32, so parameters, losses and gradients
are compared with the float64 oracle to a relative 1e-4 of their largest
magnitude; eigenvalues to 1e-6 MeV (the solves' target).
"""
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle
from oracle import mlp

FP32_REL = 1e-4
EIG_TOL = 1e-6


def _problem(seed, n=64, n_in=4, n_out=8):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, n_in))
    A = rng.standard_normal((n_in, n_out))
    t = np.sin(x @ A) + 0.1 * (x ** 2).sum(1, keepdims=True)
    return x.astype(np.float32), t.astype(np.float32)


@pytest.mark.gpu
def test_initial_parameters_match_the_oracle():
    net = jn.MLP(4, 32, 8, seed=11)
    assert np.array_equal(net.params(), mlp.init_params(4, 32, 8, 11))
    net.close()


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(4, 32, 8), (3, 128, 32), (5, 17, 3)])
def test_forward_loss_and_gradient_match_the_oracle(shape):
    n_in, h, n_out = shape
    x, t = _problem(1, n_in=n_in, n_out=n_out)
    net = jn.MLP(n_in, h, n_out, seed=5)
    p = net.params()
    y = net.predict(x)
    y_ref, _ = mlp.forward(p, x, n_in, h, n_out)
    assert np.abs(y - y_ref).max() <= FP32_REL * np.abs(y_ref).max()
    loss, g = net.loss_and_gradient(x, t)
    loss_ref, g_ref = mlp.loss_and_gradient(p, x, t, n_in, h, n_out)
    assert abs(loss - loss_ref) <= FP32_REL * loss_ref
    assert np.abs(g - g_ref).max() <= FP32_REL * np.abs(g_ref).max()
    net.close()


@pytest.mark.gpu
def test_adam_steps_follow_the_oracle():
    n_in, h, n_out = 4, 32, 8
    x, t = _problem(2, n_in=n_in, n_out=n_out)
    net = jn.MLP(n_in, h, n_out, seed=9)
    p0 = net.params()
    net.train(x, t, steps=20, learning_rate=1e-3)
    p_ref = mlp.adam(p0, x, t, n_in, h, n_out, 20, 1e-3)
    # Adam normalises each gradient component, so a component near zero may
    # step either way in FP32: compare the loss reached and the displacement of
    # all but the flattest 1 % of the parameters
    p1 = net.params()
    l1, l_ref = mlp.loss(p1, x, t, n_in, h, n_out), mlp.loss(p_ref, x, t, n_in, h, n_out)
    assert abs(l1 - l_ref) <= 1e-3 * l_ref
    dp, dp_ref = p1 - p0, p_ref - p0
    close = np.abs(dp - dp_ref) <= 1e-2 * np.abs(dp_ref).max()
    assert close.mean() >= 0.99
    net.close()


@pytest.mark.gpu
def test_training_reduces_the_loss_and_repeats_bit_for_bit():
    x, t = _problem(3)
    nets = [jn.MLP(4, 64, 8, seed=1) for _ in range(2)]
    before = nets[0].loss_and_gradient(x, t)[0]
    after = [n.train(x, t, steps=1500, learning_rate=3e-3) for n in nets]
    assert after[0] < 0.05 * before
    assert after[0] == after[1]
    assert np.array_equal(nets[0].params(), nets[1].params())
    assert abs(after[0] - mlp.loss(nets[0].params(), x, t, 4, 64, 8)) <= FP32_REL * before
    for n in nets:
        n.close()


@pytest.mark.gpu
def test_mlp_rejects_bad_sizes():
    with pytest.raises(jn.JnError):
        jn.MLP(0, 8, 8)
    with pytest.raises(jn.JnError):
        jn.MLP(4, 2048, 8)


def _dense(d):
    P = oracle.Port(d)
    D = P.dimension
    H = np.zeros((D, D))
    for i in range(D):
        e = np.zeros(D)
        e[i] = 1.0
        H[:, i] = P.matvec(e)
    return H


@pytest.fixture(scope="module")
def coupling_family(tmp_path_factory):
    """He4 Nmax 4 two-body: H(c) = H0 + sum_{i=1..4} c_i H_i on one set of lists."""
    root = tmp_path_factory.mktemp("warm")
    dirs = [str(root / f"h{i}") for i in range(5)]
    jn.generate(dirs[0], Z=2, N=2, nmax=4, nbody=2, basis_files=False)
    for i in range(1, 5):
        jn.generate(dirs[i], Z=2, N=2, nmax=4, nbody=2, seed=20261203 + 1000 * i, hbar_omega=0.0,
                    basis_files=False)
    return dirs, [_dense(d) for d in dirs]


@pytest.mark.gpu
def test_warm_start_gains_over_the_default_start(coupling_family):
    """Train on 128 solves the batched solver produced, then solve 16 held-out
    Hamiltonians from the default start vector and from the network's start
    vectors.  Both reach the dense eigenvalues; the network's start vectors
    lie mostly in the wanted eigenspace, and the solves take fewer steps."""
    dirs, dense = coupling_family
    rng = np.random.default_rng(20261203)
    S, n_test = 128, 16
    cs = rng.uniform(-1, 1, (S + n_test, 4))
    H = jn.Hamiltonian.from_dir(dirs[0], 2, 2)
    try:
        comps = [H.read_matrix_elements(os.path.join(d, "matrix_elements")) for d in dirs]
        mes = [comps[0] + sum(c[i] * comps[i + 1] for i in range(4)) for c in cs]
        _, vecs = H.lanczos_batch(mes[:S], num_eigenvalues=10, tolerance=1e-6, eigenvectors=10)
        ws = jn.WarmStart(cs[:S], vecs, hidden=128, basis_size=32, train_steps=3000, seed=0)
        B = ws.basis()
        assert np.abs(B @ B.T - np.eye(len(B))).max() < 1e-10
        starts = ws.start_vectors(cs[S:])
        cold = H.lanczos_batch(mes[S:], num_eigenvalues=10, tolerance=1e-6, check_every=1)
        warm = H.lanczos_batch(mes[S:], start_vectors=starts, num_eigenvalues=10, tolerance=1e-6, check_every=1)
        ws.close()
    finally:
        H.close()
    r = mlp.default_start_vector(len(starts[0]))
    in_space_warm, in_space_cold = [], []
    for j in range(n_test):
        Hc = dense[0] + sum(cs[S + j][i] * dense[i + 1] for i in range(4))
        w, V = np.linalg.eigh(Hc)
        for res in (cold[j], warm[j]):
            assert res["converged"]
            assert np.abs(res["eigenvalues"] - w[:10]).max() < EIG_TOL
        P = V[:, :10]
        in_space_warm.append(np.linalg.norm(P.T @ starts[j]) / np.linalg.norm(starts[j]))
        in_space_cold.append(np.linalg.norm(P.T @ r) / np.linalg.norm(r))
    it_cold = np.array([c["iterations"] for c in cold])
    it_warm = np.array([c["iterations"] for c in warm])
    print(f"\nwanted-eigenspace weight of the start vector: default {np.mean(in_space_cold):.3f}, "
          f"network {np.mean(in_space_warm):.3f}; mean Lanczos steps: default {it_cold.mean():.1f}, "
          f"network {it_warm.mean():.1f} (fewer in {(it_warm < it_cold).sum()} of {n_test})")
    assert np.mean(in_space_warm) > 0.7 > 5 * np.mean(in_space_cold)
    assert it_warm.mean() < it_cold.mean()
    assert (it_warm < it_cold).sum() > n_test // 2


@pytest.mark.gpu
def test_warm_start_rejects_bad_arguments(coupling_family):
    with pytest.raises(jn.JnError):
        jn.WarmStart(np.zeros((1, 4)), [np.ones((1, 10))], noise=-1.0)
    # snapshots orthogonal to the start vector carry no target
    with pytest.raises(jn.JnError):
        jn.WarmStart(np.zeros((1, 4)), [np.zeros((1, 10))])
