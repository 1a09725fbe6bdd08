"""Build and bind the C restatement of the reference's CPU mul! (oracle/kf_apply_ref.c).

Test infrastructure only: the fast path of the oracle's `KronFreeOperator.matvec` for real
operators, and the CPU baseline `bench.py --impl reference` times.  Built with gcc -O3 -fopenmp
into oracle/_build/ (git-ignored; rebuilt on the GPU machine by `__graft_entry__.build()`).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from . import kfref

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "kf_apply_ref.c")
OUT = os.path.join(HERE, "_build", "libkfref.so")


class _Factor(C.Structure):
    _fields_ = [("axis", C.c_int32), ("kind", C.c_int32), ("n", C.c_int64), ("data", C.POINTER(C.c_double)),
                ("offsets", C.POINTER(C.c_int64)), ("nbands", C.c_int32), ("shift", C.c_int64),
                ("factor", C.c_double)]


def build(force=False):
    if force or not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", SRC, "-o", OUT + ".tmp"])
        os.replace(OUT + ".tmp", OUT)
    return OUT


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.kf_ref_apply.restype = C.c_int
        _lib.kf_ref_resid.restype = C.c_int
        _lib.kf_ref_scale.restype = C.c_int
        _lib.kf_ref_gram.restype = C.c_int
        _lib.kf_ref_update.restype = C.c_int
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ld(a):
    """Leading dimension of an F-contiguous (N, k) block (or of a column slice of one)."""
    return a.strides[1] // 8 if a.ndim == 2 and a.shape[1] > 1 else a.shape[0]


def resid(X, HX, lam, R):
    """R = HX - X diag(lam) into the F-ordered R (threaded); returns the squared column norms."""
    N, k = X.shape
    n2 = np.empty(max(k, 1))
    for a in (X, HX, R):
        assert a.flags.f_contiguous or k == 1
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    rc = lib().kf_ref_resid(C.c_int64(N), k, _dp(X), C.c_int64(_ld(X)), _dp(HX), C.c_int64(_ld(HX)), _dp(lam),
                            _dp(R), C.c_int64(_ld(R)), _dp(n2))
    if rc:
        raise RuntimeError("kf_ref_resid failed")
    return n2[:k]


def _fcols(a):
    """True when a is a column-major (N, k) block whose columns may be strided by a leading dimension."""
    return a.ndim == 2 and a.strides[0] == 8 and (a.shape[1] <= 1 or a.strides[1] >= 8 * a.shape[0])


def gram(A, B):
    """A' B for tall column-major blocks (threaded, fixed-order partial sums)."""
    N, ka = A.shape
    kb = B.shape[1]
    G = np.empty((ka, kb), order="F")
    rc = lib().kf_ref_gram(C.c_int64(N), ka, _dp(A), C.c_int64(_ld(A)), kb, _dp(B), C.c_int64(_ld(B)), _dp(G))
    if rc:
        raise RuntimeError("kf_ref_gram failed")
    return G


def update(X, Cm, alpha=1.0, beta=0.0, Y=None):
    """Y = alpha X Cm + beta Y for a tall column-major X (threaded); a new F block when Y is None."""
    N, kx = X.shape
    Cm = np.asfortranarray(Cm, dtype=np.float64)
    ky = Cm.shape[1]
    if Y is None:
        Y = np.empty((N, ky), order="F")
        beta = 0.0
    rc = lib().kf_ref_update(C.c_int64(N), kx, _dp(X), C.c_int64(_ld(X)), ky, _dp(Cm), C.c_int64(max(Cm.shape[0], 1)),
                             C.c_double(alpha), C.c_double(beta), _dp(Y), C.c_int64(_ld(Y)))
    if rc:
        raise RuntimeError("kf_ref_update failed")
    return Y


def scale(R, S, thp, eta, mode, W):
    """W[:, j] = R[:, j] / hypot(S - thp[j], eta) (mode 0) or / (S - thp[0]) (mode 1); W may be R."""
    N, k = R.shape
    thp = np.ascontiguousarray(thp, dtype=np.float64)
    S = np.ascontiguousarray(S, dtype=np.float64)
    rc = lib().kf_ref_scale(C.c_int64(N), k, _dp(R), C.c_int64(_ld(R)), _dp(S), _dp(thp), C.c_double(eta), mode,
                            _dp(W), C.c_int64(_ld(W)))
    if rc:
        raise RuntimeError("kf_ref_scale failed")
    return W


class CApply:
    """The packed form of a real `kfref.KronFreeOperator` for kf_ref_apply."""

    def __init__(self, H):
        if H.dtype != np.float64:
            raise TypeError("CApply: real operators only")
        self.H = H
        self.keep = []
        facs, coeff, first, nf = [], [], [], []
        for c, fs in H.terms:
            first.append(len(facs))
            nf.append(len(fs))
            coeff.append(float(c))
            for a, op in fs:
                f = _Factor()
                f.axis, f.n = a, op.n
                if isinstance(op, kfref.DiagonalOp):
                    d = np.ascontiguousarray(op.d, dtype=np.float64)
                    self.keep.append(d)
                    f.kind, f.data = 0, d.ctypes.data_as(C.POINTER(C.c_double))
                elif isinstance(op, kfref.BandedOp):
                    w = np.ascontiguousarray(np.concatenate(op.weights) if op.weights else np.zeros(1), dtype=np.float64)
                    o = np.ascontiguousarray(op.offsets if op.offsets else [0], dtype=np.int64)
                    self.keep += [w, o]
                    f.kind, f.data, f.offsets, f.nbands = 1, w.ctypes.data_as(C.POINTER(C.c_double)), \
                        o.ctypes.data_as(C.POINTER(C.c_int64)), len(op.offsets)
                elif isinstance(op, kfref.ShiftOp):
                    f.kind, f.shift, f.factor = 2, op.s, float(np.real(op.factor))
                else:
                    M = np.asfortranarray(op.M, dtype=np.float64)
                    self.keep.append(M)
                    f.kind, f.data = 3, M.ctypes.data_as(C.POINTER(C.c_double))
                facs.append(f)
        self.facs = (_Factor * max(len(facs), 1))(*facs)
        self.coeff = np.array(coeff + [0.0], dtype=np.float64)
        self.first = np.array(first + [0], dtype=np.int32)
        self.nf = np.array(nf + [0], dtype=np.int32)
        self.nterms = len(coeff)
        self.dims = np.array(H.dims, dtype=np.int64)
        self.diag = np.ascontiguousarray(np.real(H.diag), dtype=np.float64)
        self.scratch = np.empty(0)

    def matvec(self, X):
        X = np.asarray(X, dtype=np.float64)
        vec = X.ndim == 1
        Xm = np.asfortranarray(X.reshape(self.H.N, -1))
        b = Xm.shape[1]
        if self.scratch.size < 2 * self.H.N * b:
            self.scratch = np.empty(2 * self.H.N * b)
        Y = np.empty_like(Xm, order="F")
        P = lambda a, t=C.c_double: a.ctypes.data_as(C.POINTER(t))
        rc = lib().kf_ref_apply(len(self.dims), P(self.dims, C.c_int64), P(self.diag), self.nterms, P(self.coeff),
                                P(self.first, C.c_int32), P(self.nf, C.c_int32), self.facs, P(Xm), P(Y),
                                C.c_int64(b), P(self.scratch))
        if rc:
            raise RuntimeError("kf_ref_apply failed")
        return Y[:, 0] if vec else Y
