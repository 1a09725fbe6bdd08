"""The learned warm start's network (libkfgpu's kf_mlp_*): din -> hidden -> hidden -> dout with SiLU,
BF16 weights, FP32 accumulation and Adam, trained and evaluated by the library's own kernels."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._abi import check, lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class MLP:
    def __init__(self, din, hidden, dout, seed=0):
        self.din, self.h, self.dout = int(din), int(hidden), int(dout)
        h = C.c_void_p()
        check(lib().kf_mlp_create(self.din, self.h, self.dout, int(seed), C.byref(h)))
        self._h = h

    def close(self):
        if self._h is not None and self._h.value:
            lib().kf_mlp_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scaling(self, xmu, xsd, ymu, ysd):
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (xmu, xsd, ymu, ysd)]
        check(lib().kf_mlp_set_scaling(self._h, *[_p(a) for a in arrs]))

    def fit_scaling(self, X, Y):
        """Standardise inputs and outputs with their sample mean and deviation."""
        xsd = np.maximum(X.std(0), 1e-12)
        ysd = np.maximum(Y.std(0), 1e-6 * max(Y.std(0).max(), 1e-12))
        self.set_scaling(X.mean(0), xsd, Y.mean(0), ysd)

    def train(self, X, Y, epochs, batch, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        losses = np.zeros(epochs, dtype=np.float32)
        check(lib().kf_mlp_train(self._h, _p(X), _p(Y), X.shape[0], int(epochs), int(batch), float(lr), int(seed),
                                 _p(losses)))
        return losses

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.empty((X.shape[0], self.dout), dtype=np.float32)
        check(lib().kf_mlp_forward(self._h, _p(X), _p(Y), X.shape[0]))
        return Y

    def gradients(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        n = C.c_int64()
        check(lib().kf_mlp_get_params(self._h, None, C.byref(n)))
        g = np.empty(n.value, dtype=np.float32)
        loss = C.c_float()
        check(lib().kf_mlp_gradients(self._h, _p(X), _p(Y), X.shape[0], C.byref(loss), _p(g)))
        return float(loss.value), g

    def params(self):
        n = C.c_int64()
        check(lib().kf_mlp_get_params(self._h, None, C.byref(n)))
        out = np.empty(n.value, dtype=np.float32)
        check(lib().kf_mlp_get_params(self._h, _p(out), C.byref(n)))
        return out

    def unpack(self, flat):
        d, h, o = self.din, self.h, self.dout
        sizes = [("W1", (d, h)), ("b1", (h,)), ("W2", (h, h)), ("b2", (h,)), ("W3", (h, o)), ("b3", (o,))]
        out, k = {}, 0
        for name, shp in sizes:
            n = int(np.prod(shp))
            out[name] = flat[k:k + n].reshape(shp)
            k += n
        return out
