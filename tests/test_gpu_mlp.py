"""The device MLP kernels of the learned guess (forward, back-propagation,
Adam) against the CPU FP64 oracle (oracle/mlp_oracle.c, itself checked
against finite differences in test_mlp_oracle.py), through the C ABI.

Tolerances: FP32 arithmetic with 16- and 64-term dot products and tanh;
outputs within 2e-5 absolute / 1e-4 relative, gradients within 1e-4 in
relative 2-norm, parameters after each Adam step (steps of about lr = 1e-3)
within 2e-5 absolute: lr g / sqrt(g^2) amplifies the FP32 error of the
smallest gradient entries."""
import numpy as np
import pytest

import feng_gb300 as fe
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _case(n, seed):
    rng = np.random.default_rng(seed)
    net = fe.MLP(seed=seed, max_batch=max(n, 1))
    dims = net.dims
    p = rng.normal(0, 0.3, net.nparams).astype(np.float32)
    net.set_params(p)
    x = rng.normal(0, 1, (n, dims[0])).astype(np.float32)
    t = rng.normal(0, 0.5, (n, dims[3])).astype(np.float32)
    m = (rng.random((n, dims[3])) > 0.25).astype(np.float32)
    return net, dims, p, x, t, m


@pytest.mark.parametrize("n", [1, 127, 128, 300, 1000])
def test_forward_matches_oracle(n):
    net, dims, p, x, _, _ = _case(n, 5)
    y = net.forward(x)
    yref = orc.mlp_forward(p.astype(np.float64), dims, x.astype(np.float64))
    np.testing.assert_allclose(y, yref, rtol=1e-4, atol=2e-5)


@pytest.mark.parametrize("n", [1, 128, 300, 1000])
def test_gradient_matches_oracle(n):
    net, dims, p, x, t, m = _case(n, 9)
    loss, g = net.train_step(x, t, m, lr=0.0)
    lref, gref = orc.mlp_loss_grad(p.astype(np.float64), dims, x.astype(np.float64), t.astype(np.float64),
                                   m.astype(np.float64))
    assert loss == pytest.approx(lref, rel=1e-4)
    assert np.linalg.norm(g - gref) <= 1e-4 * np.linalg.norm(gref)
    np.testing.assert_array_equal(net.params(), p)   # lr = 0 leaves the weights


def test_adam_steps_match_oracle():
    net, dims, p, x, t, m = _case(300, 13)
    pr = p.astype(np.float64)
    mo, vo = np.zeros_like(pr), np.zeros_like(pr)
    for step in range(1, 4):
        _, g = net.train_step(x, t, m, lr=1e-3)
        _, gref = orc.mlp_loss_grad(pr, dims, x.astype(np.float64), t.astype(np.float64), m.astype(np.float64))
        assert np.linalg.norm(g - gref) <= 1e-4 * np.linalg.norm(gref)
        pr, mo, vo = orc.mlp_adam(pr, mo, vo, gref, lr=1e-3, step=step)
        np.testing.assert_allclose(net.params(), pr, rtol=0, atol=2e-5)


def test_training_reduces_loss_on_a_linear_target():
    """A target that is a linear map of the inputs (what a second-order time
    extrapolation is): 200 full-batch Adam steps cut the loss 10x."""
    rng = np.random.default_rng(2)
    net = fe.MLP(seed=3, max_batch=2048)
    x = rng.normal(0, 1, (2048, 16)).astype(np.float32)
    a = rng.normal(0, 0.3, (16, 4)).astype(np.float32)
    t = (x @ a).astype(np.float32)
    m = np.ones_like(t)
    m[:, 3] = 0
    first, _ = net.train_step(x, t, m, lr=3e-3)
    for _ in range(200):
        last, _ = net.train_step(x, t, m, lr=3e-3)
    assert last < 0.1 * first
