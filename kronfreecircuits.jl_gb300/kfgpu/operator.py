"""KronFreeOperator on the GPU: the reference's operator interface over libkfgpu.so.

  KronFreeOperator(dims, terms; constant, block_capacity)   src/apply.jl:222-253
  mul!(Y, H, X) / H * X                                       src/apply.jl:416-435
  diagonal(H), gershgorin_bound(H)                            src/apply.jl:455, 586-593
  separable_eigenbases(H), product_seed(H, k)                 src/apply.jl:606-685 (host, as in the reference)

`terms` is a list of (coeff, [(axis, op), ...]) with 0-based strictly increasing axes and ops
from `kfgpu.ops`.  The operator data is copied to the current CUDA device at construction.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import check, lib
from .ops import BandedOp, DenseOp, DiagonalOp, ShiftOp


def _ptr(a, typ=C.c_double):
    return a.ctypes.data_as(C.POINTER(typ))


class _Desc:
    """A kf_op_desc plus the arrays it points into (kept alive while the descriptor is used)."""

    def __init__(self, dims, terms, constant=0.0, block_capacity=1, diag=None):
        self.keep = []
        self.dims = np.ascontiguousarray(dims, dtype=np.int64)
        cterms = (_abi.KfTerm * max(len(terms), 1))()
        for t, (coeff, factors) in enumerate(terms):
            cf = (_abi.KfFactor * max(len(factors), 1))()
            for k, (axis, op) in enumerate(factors):
                f = cf[k]
                f.axis, f.n = int(axis), int(op.n)
                if isinstance(op, DiagonalOp):
                    f.kind = _abi.KF_DIAG
                    d = np.ascontiguousarray(op.d, dtype=np.float64)
                    self.keep.append(d)
                    f.data = _ptr(d)
                elif isinstance(op, BandedOp):
                    f.kind = _abi.KF_BANDED
                    w = np.ascontiguousarray(np.concatenate(op.weights) if op.weights else np.zeros(1))
                    o = np.ascontiguousarray(op.offsets if op.offsets else [0], dtype=np.int64)
                    self.keep += [w, o]
                    f.data, f.offsets, f.nbands = _ptr(w), _ptr(o, C.c_int64), len(op.offsets)
                elif isinstance(op, ShiftOp):
                    f.kind, f.shift, f.factor = _abi.KF_SHIFT, op.s, op.factor
                elif isinstance(op, DenseOp):
                    f.kind = _abi.KF_DENSE
                    M = np.asfortranarray(op.M, dtype=np.float64)
                    self.keep.append(M)
                    f.data = _ptr(M)
                else:
                    raise TypeError(f"unsupported factor {type(op).__name__}")
            self.keep.append(cf)
            cterms[t].coeff, cterms[t].nfactors = float(coeff), len(factors)
            cterms[t].factors = C.cast(cf, C.POINTER(_abi.KfFactor))
        self.keep.append(cterms)
        self.desc = _abi.KfOpDesc()
        self.desc.ndims = len(self.dims)
        self.desc.dims = _ptr(self.dims, C.c_int64)
        self.desc.constant = float(constant)
        self.desc.nterms = len(terms)
        self.desc.terms = C.cast(cterms, C.POINTER(_abi.KfTerm))
        if diag is not None:
            dg = np.ascontiguousarray(diag, dtype=np.float64)
            self.keep.append(dg)
            self.desc.diag = _ptr(dg)
        self.desc.block_capacity = int(block_capacity)


class KronFreeOperator:
    def __init__(self, dims, terms, constant=0.0, block_capacity=1, diag=None):
        self.dims = [int(d) for d in dims]
        self.terms = list(terms)
        self.constant = float(constant)
        self.N = int(np.prod(self.dims))
        self._h = None
        d = _Desc(self.dims, self.terms, constant, block_capacity, diag)
        h = C.c_void_p()
        check(lib().kf_op_create(C.byref(d.desc), C.byref(h)))
        self._h = h

    # -- lifecycle
    def close(self):
        if self._h is not None and self._h.value:
            lib().kf_op_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def shape(self):
        return (self.N, self.N)

    # -- application
    def apply(self, X, f32=False):
        """H X for a host block (N or N x b), through the library's host path (copies in and out)."""
        dt = np.float32 if f32 else np.float64
        X = np.asarray(X, dtype=dt)
        vec = X.ndim == 1
        Xm = np.asfortranarray(X.reshape(self.N, -1) if vec else X)
        if Xm.shape[0] != self.N:
            raise _abi.DimensionMismatch(_abi.KF_EDIM, f"KronFreeOperator of size {self.shape} applied to x with {Xm.shape[0]} rows")
        Y = np.empty_like(Xm, order="F")
        flags = _abi.KF_HOST | (_abi.KF_F32 if f32 else _abi.KF_F64)
        check(lib().kf_op_apply(self._h, Xm.ctypes.data, Y.ctypes.data, self.N, self.N, Xm.shape[1], flags))
        return Y[:, 0] if vec else Y

    __matmul__ = apply

    def apply_device(self, x_ptr, y_ptr, b, ldx=None, ldy=None, f32=False):
        """Asynchronous H X on device pointers (column-major, leading dimensions ldx, ldy)."""
        flags = _abi.KF_DEVICE | (_abi.KF_F32 if f32 else _abi.KF_F64)
        check(lib().kf_op_apply(self._h, x_ptr, y_ptr, ldx or self.N, ldy or self.N, b, flags))

    def apply_axpby_device(self, x_ptr, y_ptr, z_ptr, b, alpha, beta, gamma, f32=False):
        flags = _abi.KF_F32 if f32 else _abi.KF_F64
        check(lib().kf_op_apply_axpby(self._h, x_ptr, y_ptr, z_ptr, self.N, b, alpha, beta, gamma, flags))

    def sync(self):
        check(lib().kf_op_sync(self._h))

    def stream(self):
        s = C.c_void_p()
        check(lib().kf_op_get_stream(self._h, C.byref(s)))
        return s.value

    def set_stream(self, stream_ptr):
        check(lib().kf_op_set_stream(self._h, C.c_void_p(stream_ptr)))

    # -- derived quantities
    def diagonal(self):
        out = np.empty(self.N)
        check(lib().kf_op_diagonal(self._h, _ptr(out)))
        return out

    def gershgorin_bound(self):
        v = C.c_double()
        check(lib().kf_op_gershgorin(self._h, C.byref(v)))
        return v.value

    def separable_eigenbases(self):
        """Per axis, the eigenbasis of the sum of single-axis terms (src/apply.jl:606-642); host data."""
        A = [np.zeros((d, d)) for d in self.dims]
        for c, fs in self.terms:
            if len(fs) == 1:
                a, op = fs[0]
                A[a] += c * op.dense()
        A[0] += self.constant * np.eye(self.dims[0])
        U, lam = [], []
        for M in A:
            if not np.any(M - np.diag(np.diag(M))):
                U.append(None)
                lam.append(np.diag(M).copy())
            else:
                w, V = np.linalg.eigh((M + M.T) / 2)
                U.append(V)
                lam.append(w)
        return U, lam

    def product_seed_device(self, k):
        """product_seed(H, k) built by the library on the device (kf_op_product_seed), host N x k."""
        X = np.empty((self.N, k), order="F")
        check(lib().kf_op_product_seed(self._h, int(k), X.ctypes.data, _abi.KF_HOST))
        return X

    def product_seed(self, k):
        """k orthonormal lowest product states (src/apply.jl:655-685), host N x k."""
        if not 1 <= k <= self.N:
            raise _abi.ArgumentError(_abi.KF_EINVAL, f"product_seed: k must lie in 1:{self.N}, got {k}")
        U, lam = self.separable_eigenbases()
        X = np.zeros((self.N, k), order="F")
        if all(u is None for u in U):
            idx = np.argsort(self.diagonal(), kind="stable")[:k]
            X[idx, np.arange(k)] = 1.0
            return X
        sums = lam[0]
        for a in range(1, len(self.dims)):
            sums = (sums[:, None] + lam[a][None, :]).reshape(-1, order="F")
        for j, flat in enumerate(np.argsort(sums, kind="stable")[:k]):
            idx = np.unravel_index(flat, self.dims, order="F")
            v = np.ones(1)
            for a in range(len(self.dims)):
                ua = np.eye(self.dims[a])[:, idx[a]] if U[a] is None else U[a][:, idx[a]]
                v = np.kron(ua, v)
            X[:, j] = v
        return X
