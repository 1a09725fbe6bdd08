"""The warm-start network's hand-written kernels against the NumPy reference (oracle/mlp.py):
forward pass, loss and every parameter gradient (FP32 on the GPU vs FP64 on the host, same BF16
weights), and an Adam training run that reduces the loss on a smooth synthetic target."""
import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradients_match_numpy(cuda):
    from kfgpu.mlp import MLP
    rng = np.random.default_rng(0)
    din, h, dout, n = 7, 64, 96, 200
    net = MLP(din, h, dout, seed=3)
    X = rng.uniform(-1, 1, (n, din)).astype(np.float32)
    Y = np.sin(X @ rng.standard_normal((din, dout))).astype(np.float32)
    xmu, xsd = X.mean(0), X.std(0)
    ymu, ysd = Y.mean(0), Y.std(0) + 1e-3
    net.set_scaling(xmu, xsd, ymu, ysd)
    P = net.unpack(net.params())
    out_ref, _ = omlp.forward({k: v.astype(np.float64) for k, v in P.items()}, X, xmu, xsd)
    out = net.forward(X)
    assert np.max(np.abs(out - (out_ref * ysd + ymu))) < 1e-3 * max(1.0, np.abs(out).max())
    loss, g = net.gradients(X, Y)
    loss_ref, g_ref = omlp.loss_and_grads(P, X, Y, xmu, xsd, ymu, ysd)
    assert abs(loss - loss_ref) < 1e-4 * loss_ref
    G = net.unpack(g)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        rel = np.max(np.abs(G[k] - g_ref[k])) / max(np.max(np.abs(g_ref[k])), 1e-12)
        assert rel < 2e-3, (k, rel)


def test_mlp_training_reduces_loss(cuda):
    from kfgpu.mlp import MLP
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, (2048, 7)).astype(np.float32)
    Y = np.tanh(X @ rng.standard_normal((7, 32))).astype(np.float32)
    net = MLP(7, 128, 32, seed=5)
    net.fit_scaling(X, Y)
    losses = net.train(X, Y, epochs=30, batch=256, lr=2e-3, seed=2)
    assert losses[-1] < 0.1 * losses[0], losses[[0, -1]]
