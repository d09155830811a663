"""MLP oracle — TEST INFRASTRUCTURE ONLY.

A numpy restatement, in float64, of the learned warm start's network
(include/jncsm.h, "Learned warm start"): forward pass, loss, analytic
gradient by back-propagation and the Adam update.  The GPU kernels are
checked against it.  The reference has no counterpart; the parameter layout
and the loss are the ones the C ABI documents.

Layout of the flat parameter vector: W1 (H x n_in), b1 (H), W2 (H x H),
b2 (H), W3 (n_out x H), b3 (n_out), row-major with the output index first.
"""
import math

import numpy as np

_erf = np.vectorize(math.erf, otypes=[np.float64])


def unpack(p, n_in, h, n_out):
    p = np.asarray(p, dtype=np.float64)
    sizes = [h * n_in, h, h * h, h, n_out * h, n_out]
    assert len(p) == sum(sizes), (len(p), sum(sizes))
    parts, o = [], 0
    for s in sizes:
        parts.append(p[o:o + s])
        o += s
    W1, b1, W2, b2, W3, b3 = parts
    return W1.reshape(h, n_in), b1, W2.reshape(h, h), b2, W3.reshape(n_out, h), b3


def gelu(a):
    return 0.5 * a * (1.0 + _erf(a / math.sqrt(2.0)))


def gelu_grad(a):
    return 0.5 * (1.0 + _erf(a / math.sqrt(2.0))) + a * np.exp(-0.5 * a * a) / math.sqrt(2.0 * math.pi)


def forward(p, x, n_in, h, n_out):
    """Returns y and the activations (a1, h1, a2, h2)."""
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, h, n_out)
    x = np.asarray(x, dtype=np.float64)
    a1 = x @ W1.T + b1
    h1 = gelu(a1)
    a2 = h1 @ W2.T + b2
    h2 = gelu(a2)
    y = h2 @ W3.T + b3
    return y, (a1, h1, a2, h2)


def loss(p, x, t, n_in, h, n_out):
    y, _ = forward(p, x, n_in, h, n_out)
    return float(((y - np.asarray(t, dtype=np.float64)) ** 2).sum() / (2 * len(y)))


def loss_and_gradient(p, x, t, n_in, h, n_out):
    """Loss sum_s |y_s - t_s|^2 / (2 n) and its gradient, by back-propagation."""
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, h, n_out)
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    y, (a1, h1, a2, h2) = forward(p, x, n_in, h, n_out)
    e = y - np.asarray(t, dtype=np.float64)
    d3 = e / n
    d2 = (d3 @ W3) * gelu_grad(a2)
    d1 = (d2 @ W2) * gelu_grad(a1)
    g = np.concatenate([(d1.T @ x).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0),
                        (d3.T @ h2).ravel(), d3.sum(0)])
    return float((e ** 2).sum() / (2 * n)), g


def adam(p, x, t, n_in, h, n_out, steps, lr, b1=0.9, b2=0.999, eps=1e-8):
    """`steps` full-batch Adam steps from p; returns the final parameters."""
    p = np.array(p, dtype=np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for k in range(1, steps + 1):
        _, g = loss_and_gradient(p, x, t, n_in, h, n_out)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p = p - lr * (m / (1 - b1 ** k)) / (np.sqrt(v / (1 - b2 ** k)) + eps)
    return p


def init_params(n_in, h, n_out, seed):
    """The initialisation jn_mlp_create uses: SplitMix64 uniforms in [-1, 1)
    scaled by 1/sqrt(fan_in) for the weights, zero biases (rounded to FP32)."""
    M = (1 << 64) - 1
    z = seed & M

    def unif():
        nonlocal z
        z = (z + 0x9E3779B97F4A7C15) & M
        v = z
        v = ((v ^ (v >> 30)) * 0xBF58476D1CE4E5B9) & M
        v = ((v ^ (v >> 27)) * 0x94D049BB133111EB) & M
        v ^= v >> 31
        return (v >> 11) * 2.0 ** -53 * 2.0 - 1.0

    W1 = [unif() / math.sqrt(n_in) for _ in range(h * n_in)]
    W2 = [unif() / math.sqrt(h) for _ in range(h * h)]
    W3 = [unif() / math.sqrt(h) for _ in range(n_out * h)]
    p = np.concatenate([W1, np.zeros(h), W2, np.zeros(h), W3, np.zeros(n_out)])
    return p.astype(np.float32)


def default_start_vector(dim):
    """The batched solver's default start vector: SplitMix64 uniforms in [-0.5, 0.5)."""
    M = (1 << 64) - 1
    z = 0x9E3779B97F4A7C15
    out = np.empty(dim)
    for e in range(dim):
        z = (z + 0x9E3779B97F4A7C15) & M
        v = z
        v = ((v ^ (v >> 30)) * 0xBF58476D1CE4E5B9) & M
        v = ((v ^ (v >> 27)) * 0x94D049BB133111EB) & M
        v ^= v >> 31
        out[e] = (v >> 11) * 2.0 ** -53 - 0.5
    return out


def warm_start_targets(eigenvectors, r):
    """u_s = sum_e v_e (v_e . r) / |.| for each sample's eigenvectors (k x D)."""
    out = []
    for V in eigenvectors:
        u = V.T @ (V @ r)
        out.append(u / np.linalg.norm(u))
    return np.array(out)
