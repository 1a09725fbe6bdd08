"""The linear solve on the complement of a node's known states, on the GPU (kf_complement_solve).

  complement_solve(H, basis, B, shifts, tol, maxiter; eta, scale)   src/resolvent.jl:146-252

Mirrors the reference's `_complement_solve(H, D, basis, B, shifts; tol, maxiter, eta, scale)`:
X[:, j] solves Q (H - shifts[j]) Q x = Q B[:, j] with x orthogonal to the orthonormal columns of
`basis` (Q = 1 - basis basis'), by a Jacobi-preconditioned conjugate gradient on all columns in
lockstep; D is H's own diagonal.  Returns (X, iterations, residuals, from_start, at_floor,
floor_residuals) with 0-based column indices.  Errors: ConvergenceError with "not positive on the
complement" (KF_EBREAKDOWN) or "did not converge" (KF_ENOCONV), as the reference's error().
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi


def complement_solve(H, basis, B, shifts, tol, maxiter, eta=0.01, scale=None):
    Bf = np.asfortranarray(B, dtype=np.float64)
    if Bf.ndim != 2 or Bf.shape[0] != H.N:
        raise _abi.DimensionMismatch(_abi.KF_EDIM, f"complement_solve: B has shape {Bf.shape}, expected ({H.N}, n)")
    n = Bf.shape[1]
    sh = np.ascontiguousarray(shifts, dtype=np.float64)
    if sh.shape != (n,):
        raise _abi.DimensionMismatch(_abi.KF_EDIM, f"{n} columns and {sh.size} shifts")
    sc = None
    if scale is not None:
        sc = np.ascontiguousarray(scale, dtype=np.float64)
        if sc.shape != (n,):
            raise _abi.DimensionMismatch(_abi.KF_EDIM, f"{n} columns and {sc.size} scales")
    V = np.asfortranarray(basis, dtype=np.float64) if basis is not None else np.zeros((H.N, 0), order="F")
    if V.ndim != 2 or V.shape[0] != H.N:
        raise _abi.DimensionMismatch(_abi.KF_EDIM, f"complement_solve: basis has shape {V.shape}, expected ({H.N}, k)")
    X = np.empty((H.N, n), order="F")
    it = C.c_int32(0)
    state = np.zeros(n, dtype=np.int32)
    res = np.zeros(n)
    fres = np.zeros(n)
    _abi.check(_abi.lib().kf_complement_solve(
        H.handle, V.ctypes.data if V.shape[1] else None, H.N, V.shape[1], Bf.ctypes.data, H.N, n, sh.ctypes.data,
        None if sc is None else sc.ctypes.data, float(tol), int(maxiter), float(eta), X.ctypes.data, H.N,
        C.byref(it), state.ctypes.data, res.ctypes.data, fres.ctypes.data, _abi.KF_HOST))
    from_start = [j for j in range(n) if state[j] == 1]
    at_floor = [j for j in range(n) if state[j] == 2]
    return X, it.value, res, from_start, at_floor, fres
