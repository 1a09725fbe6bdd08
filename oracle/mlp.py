"""NumPy reference of the warm-start MLP's forward pass, loss and gradients (test infrastructure only).

The network: x_n = (x - xmu)/xsd; A1 = SiLU(x_n W1 + b1); A2 = SiLU(A1 W2 + b2); out = A2 W3 + b3;
loss = mean((out - (y - ymu)/ysd)^2).  Computed in FP64 from the library's own parameters (the BF16
weights widened to FP32, FP32 biases), so the GPU's FP32 gradients can be compared with it.
"""
import numpy as np


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(P, X, xmu, xsd):
    xn = (X.astype(np.float64) - xmu) / xsd
    Z1 = xn @ P["W1"] + P["b1"]
    A1 = _silu(Z1)
    Z2 = A1 @ P["W2"] + P["b2"]
    A2 = _silu(Z2)
    out = A2 @ P["W3"] + P["b3"]
    return out, (xn, Z1, A1, Z2, A2)


def loss_and_grads(P, X, Y, xmu, xsd, ymu, ysd):
    P = {k: v.astype(np.float64) for k, v in P.items()}
    out, (xn, Z1, A1, Z2, A2) = forward(P, X, xmu, xsd)
    T = (Y.astype(np.float64) - ymu) / ysd
    d = out - T
    loss = np.mean(d ** 2)
    dout = 2.0 * d / d.size
    g = {"W3": A2.T @ dout, "b3": dout.sum(0)}
    dZ2 = (dout @ P["W3"].T) * _dsilu(Z2)
    g["W2"], g["b2"] = A1.T @ dZ2, dZ2.sum(0)
    dZ1 = (dZ2 @ P["W2"].T) * _dsilu(Z1)
    g["W1"], g["b1"] = xn.T @ dZ1, dZ1.sum(0)
    return loss, g
