"""The NumPy restatement of the indicator network, checked on its own: its
analytic gradient against central finite differences of its loss (float64),
and its GELU derivative against finite differences of its GELU.  The CUDA
training kernels are then checked against this restatement on the GPU."""
import numpy as np

import mlp_oracle as mo


def _batch(seed=0, n=48):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1.0, 1.0, (n, mo.N_IN))
    y = (rng.uniform(size=n) < 0.4).astype(np.float64)
    return X, y


def test_gradient_matches_finite_differences():
    X, y = _batch()
    p = mo.init_params(11).astype(np.float64)
    p[1600:1632] = np.random.default_rng(1).normal(0.0, 0.1, 32)  # non-zero biases
    p[2656:2688] = np.random.default_rng(2).normal(0.0, 0.1, 32)
    p[2720] = 0.3
    _, g = mo.loss_and_grad(p, X, y)
    rng = np.random.default_rng(3)
    # indices from every block of the layout, both ends of each block included
    blocks = [(0, 1600), (1600, 1632), (1632, 2656), (2656, 2688), (2688, 2720), (2720, 2721)]
    idx = []
    for lo, hi in blocks:
        idx += [lo, hi - 1] + list(rng.integers(lo, hi, size=min(10, hi - lo)))
    h = 1e-6
    for k in sorted(set(int(i) for i in idx)):
        e = np.zeros_like(p)
        e[k] = h
        fd = (mo.loss_and_grad(p + e, X, y)[0] - mo.loss_and_grad(p - e, X, y)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-7 + 1e-5 * abs(g[k]), (k, fd, g[k])


def test_gelu_derivative_matches_finite_differences():
    z = np.linspace(-6.0, 6.0, 241)
    h = 1e-6
    fd = (mo.gelu(z + h) - mo.gelu(z - h)) / (2 * h)
    assert np.max(np.abs(fd - mo.gelu_grad(z))) < 1e-8


def test_adam_first_step_moves_by_lr_against_the_gradient_sign():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -1e-4, 0.0])
    q, m, v = mo.adam(p, g, np.zeros(3), np.zeros(3), 1, 1e-2)
    # bias-corrected first step: m_hat = g, v_hat = g^2, so the step is lr * g / (|g| + eps)
    assert np.allclose(q[:2], p[:2] - 1e-2 * np.sign(g[:2]), atol=1e-6)
    assert q[2] == p[2]
    assert np.allclose(m, 0.1 * g) and np.allclose(v, 0.001 * g * g)


def test_loss_is_the_mean_binary_cross_entropy():
    X, y = _batch(seed=5, n=16)
    p = mo.init_params(4).astype(np.float64)
    logit, _ = mo.forward(p, X)
    pr = 1.0 / (1.0 + np.exp(-logit))
    ref = -np.mean(y * np.log(pr) + (1 - y) * np.log(1 - pr))
    loss, _ = mo.loss_and_grad(p, X, y)
    assert abs(loss - ref) < 1e-12
