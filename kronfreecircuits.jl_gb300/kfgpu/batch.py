"""Batched leaf solves over libkfgpu's kf_batch_solve: many single-axis leaves (diagonal, banded
and shift terms) in one persistent, graph-captured launch, the threads per CTA picked by the
library's autotuner (kf_batch_autotune)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import check, lib
from .operator import _Desc


def _descs(ops):
    keep = [_Desc(dims, terms, const) for dims, terms, const in ops]
    arr = (_abi.KfOpDesc * len(keep))(*[k.desc for k in keep])
    return keep, arr


def batch_solve(ops, m, tol, maxiter=200, tile=0):
    """ops: [(dims, terms, constant)]; m: per-op pair counts.  Returns (Es, Vs, iters, resid)."""
    keep, arr = _descs(ops)
    m = np.ascontiguousarray(m, dtype=np.int32)
    Ns = [int(np.prod(d)) for d, _, _ in ops]
    E = np.empty(int(m.sum()))
    V = np.empty(int(sum(n * k for n, k in zip(Ns, m))))
    iters = np.empty(len(ops), dtype=np.int32)
    resid = np.empty(len(ops))
    st = lib().kf_batch_solve(arr, len(ops), m.ctypes.data_as(C.POINTER(C.c_int32)), float(tol), int(maxiter), int(tile),
                              E.ctypes.data, V.ctypes.data, iters.ctypes.data, resid.ctypes.data)
    Es, Vs, eo, vo = [], [], 0, 0
    for n, k in zip(Ns, m):
        Es.append(E[eo:eo + k])
        Vs.append(V[vo:vo + n * k].reshape((n, k), order="F"))
        eo += k
        vo += n * k
    if st != _abi.KF_OK:
        try:
            check(st)
        except _abi.KFError as e:
            e.partial = (Es, Vs, iters, resid)
            raise
    return Es, Vs, iters, resid


def autotune(ops, m, tol, maxiter=200):
    keep, arr = _descs(ops)
    m = np.ascontiguousarray(m, dtype=np.int32)
    best = C.c_int32()
    check(lib().kf_batch_autotune(arr, len(ops), m.ctypes.data_as(C.POINTER(C.c_int32)), float(tol), int(maxiter),
                                  C.byref(best)))
    return best.value
