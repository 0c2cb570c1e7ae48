"""The learned models' network on the GPU against its CPU restatement
(oracle/mlp_ref.py, float64): forward pass, gradient, one Adam step, and that
training reduces the loss."""
import numpy as np
import pytest

from oracle import mlp_ref as R

pytestmark = pytest.mark.gpu

D, H1, H2 = 10, 32, 32


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, D)).astype(np.float32)
    w = rng.standard_normal(D)
    y = (np.tanh(X @ w / 3.0) + 0.1 * X[:, 0] ** 2).astype(np.float32)
    return X, y


def test_forward_matches_cpu(gpu_lib):
    net = gpu_lib.MLP(D, H1, H2, seed=3)
    X, _ = _data(777, 1)
    out = net.predict(X)
    ref, _ = R.forward(net.params(), X, D, H1, H2)
    assert np.allclose(out, ref, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("n", [1, 100, 1000])
def test_gradient_matches_cpu(gpu_lib, n):
    net = gpu_lib.MLP(D, H1, H2, seed=5)
    X, y = _data(n, 2)
    loss, g = net.gradient(X, y)
    lr, gr = R.loss_and_grad(net.params(), X, y, D, H1, H2)
    assert abs(loss - lr) <= 1e-5 * max(1.0, abs(lr))
    assert np.linalg.norm(g - gr) <= 1e-4 * np.linalg.norm(gr)
    assert np.abs(g - gr).max() <= 1e-4 * np.abs(gr).max()


def test_adam_step_matches_cpu(gpu_lib):
    net = gpu_lib.MLP(D, H1, H2, seed=7)
    X, y = _data(512, 3)
    p0 = net.params().astype(np.float64)
    net.train(X, y, epochs=1, batch=512, lr=1e-2, seed=0)  # one step over all samples
    _, g = R.loss_and_grad(p0, X, y, D, H1, H2)
    p1, _, _ = R.adam(p0, np.zeros_like(p0), np.zeros_like(p0), g, 1, 1e-2)
    assert np.allclose(net.params(), p1, rtol=0, atol=2e-5)


def test_training_reduces_loss(gpu_lib):
    net = gpu_lib.MLP(D, H1, H2, seed=11)
    X, y = _data(4096, 4)
    l0, _ = net.gradient(X, y)
    l1 = net.train(X, y, epochs=40, batch=256, lr=3e-3, seed=1)
    assert l1 < 0.1 * l0
    # deterministic: the same seeds give the same parameters
    net2 = gpu_lib.MLP(D, H1, H2, seed=11)
    net2.train(X, y, epochs=40, batch=256, lr=3e-3, seed=1)
    assert np.array_equal(net.params(), net2.params())


def test_params_roundtrip_and_errors(gpu_lib):
    net = gpu_lib.MLP(D, H1, H2, seed=1)
    p = net.params()
    assert p.size == H1 * D + H1 + H2 * H1 + 2 * H2 + 1
    other = gpu_lib.MLP(D, H1, H2, seed=2)
    other.set_params(p)
    assert np.array_equal(other.params(), p)
    with pytest.raises(gpu_lib.MCBError):
        gpu_lib.MLP(0, H1, H2)
    with pytest.raises(gpu_lib.MCBError):
        gpu_lib.MLP(D, 64, H2)
