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
    return _lib


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
