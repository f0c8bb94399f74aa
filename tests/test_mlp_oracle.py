"""The CPU FP64 oracle of the learned-guess MLP: back-propagated gradients
against central finite differences, and Adam's known first-step answer.
These pin the oracle that the device MLP kernels are checked against."""
import numpy as np
import pytest

from oracle import oracle as orc

DIMS = (16, 64, 64, 4)


def _setup(seed=3, n=37):
    rng = np.random.default_rng(seed)
    npar = orc.mlp_param_count(DIMS)
    params = rng.normal(0, 0.3, npar)
    x = rng.normal(0, 1, (n, DIMS[0]))
    t = rng.normal(0, 0.5, (n, DIMS[3]))
    mask = (rng.random((n, DIMS[3])) > 0.25).astype(float)
    return params, x, t, mask


def test_param_count():
    assert orc.mlp_param_count(DIMS) == 64 * 16 + 64 + 64 * 64 + 64 + 4 * 64 + 4


def test_gradient_matches_finite_differences():
    params, x, t, mask = _setup()
    loss, g = orc.mlp_loss_grad(params, DIMS, x, t, mask)
    assert loss > 0
    rng = np.random.default_rng(7)
    idx = rng.choice(params.size, 60, replace=False)
    h = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += h
        p2[i] -= h
        fd = (orc.mlp_loss_grad(p1, DIMS, x, t, mask)[0] - orc.mlp_loss_grad(p2, DIMS, x, t, mask)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 * max(1.0, abs(g[i])) + 1e-9, (i, fd, g[i])


def test_masked_outputs_do_not_contribute():
    params, x, t, mask = _setup()
    t2 = t.copy()
    t2[mask == 0] += 100.0          # change only masked-out targets
    l1, g1 = orc.mlp_loss_grad(params, DIMS, x, t, mask)
    l2, g2 = orc.mlp_loss_grad(params, DIMS, x, t2, mask)
    assert l1 == pytest.approx(l2, rel=1e-14)
    np.testing.assert_allclose(g1, g2, rtol=1e-14, atol=0)


def test_forward_matches_numpy():
    params, x, _, _ = _setup()
    nin, h1, h2, nout = DIMS
    o = 0
    W1 = params[o:o + h1 * nin].reshape(h1, nin); o += h1 * nin
    b1 = params[o:o + h1]; o += h1
    W2 = params[o:o + h2 * h1].reshape(h2, h1); o += h2 * h1
    b2 = params[o:o + h2]; o += h2
    W3 = params[o:o + nout * h2].reshape(nout, h2); o += nout * h2
    b3 = params[o:o + nout]
    y = np.tanh(np.tanh(x @ W1.T + b1) @ W2.T + b2) @ W3.T + b3
    np.testing.assert_allclose(orc.mlp_forward(params, DIMS, x), y, rtol=1e-13, atol=1e-13)


def test_adam_first_step_is_lr_times_sign():
    rng = np.random.default_rng(11)
    p = rng.normal(size=50)
    g = rng.normal(size=50)
    p1, m, v = orc.mlp_adam(p, np.zeros(50), np.zeros(50), g, lr=1e-2, step=1, eps=0.0)
    np.testing.assert_allclose(p - p1, 1e-2 * np.sign(g), rtol=1e-12)
    np.testing.assert_allclose(m, 0.1 * g, rtol=1e-14)
    np.testing.assert_allclose(v, 0.001 * g * g, rtol=1e-14)
