"""The dispatcher network's CUDA kernels against the f64 oracle: forward
outputs, loss and every parameter's gradient; training with the library's
Adam kernel lowers the loss."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


def _net_and_data(n=300, seed=0):
    import torch
    from ndconv.mlp import MLP
    net = MLP(16, 64, 6, seed=seed)
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, 16))
    t = rng.standard_normal((n, 6))
    m = (rng.random((n, 6)) > 0.2).astype(np.float64)
    return net, x, t, m, torch


@pytest.mark.parametrize("n", [1, 31, 32, 33, 300])
def test_mlp_forward_and_gradient_vs_oracle(n):
    net, x, t, m, torch = _net_and_data(n)
    p = net.get_params().astype(np.float64)
    y = net.forward_raw(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    y64, _ = mlp_ref.forward(p, x.astype(np.float32), 16, 64, 6)
    assert np.abs(y - y64).max() <= 1e-4 * max(1.0, np.abs(y64).max())
    g, loss = net.gradient_raw(torch.tensor(x, dtype=torch.float32), torch.tensor(t, dtype=torch.float32),
                               torch.tensor(m, dtype=torch.float32))
    loss64, g64 = mlp_ref.loss_and_grad(p, x.astype(np.float32), t.astype(np.float32), m, 16, 64, 6)
    g = g.cpu().numpy().astype(np.float64)
    assert abs(loss - loss64) <= 1e-4 * abs(loss64)
    assert np.linalg.norm(g - g64) <= 1e-4 * np.linalg.norm(g64)
    net.close()


def test_mlp_gradient_deterministic():
    net, x, t, m, torch = _net_and_data(500, seed=3)
    args = [torch.tensor(a, dtype=torch.float32) for a in (x, t, m)]
    g1, l1 = net.gradient_raw(*args)
    g2, l2 = net.gradient_raw(*args)
    assert torch.equal(g1, g2) and l1 == l2
    net.close()


def test_mlp_training_fits_a_smooth_target():
    import torch
    from ndconv.mlp import MLP
    rng = np.random.default_rng(4)
    X = rng.standard_normal((4000, 16))
    W = rng.standard_normal((16, 6)) / 4
    T = np.sin(X @ W) + 0.1 * (X[:, :6] ** 2)
    M = np.ones_like(T)
    net = MLP(16, 64, 6, seed=1)
    args = [torch.tensor(a, dtype=torch.float32) for a in (X, T, M)]
    _, loss0 = net.gradient_raw(*args)
    loss1 = net.train_raw(*args, epochs=60, batch=128, lr=3e-3, seed=2)
    assert loss1 < 0.1 * loss0, (loss0, loss1)
    # parameters round-trip through the host
    p = net.get_params()
    net2 = MLP(16, 64, 6, seed=9)
    net2.set_params(p)
    assert torch.equal(net.forward_raw(args[0]), net2.forward_raw(args[0]))
    net.close()
    net2.close()
