"""NumPy restatement of the reference's linear solve on the complement of a node's known states
(test infrastructure only).

  src/resolvent.jl:111        _colredot: the real part of the column-wise dot products
  src/resolvent.jl:115-117    the round-off cap (1000 eps of each column's right-hand side) and the
                              floor patience (5 checks without halving)
  src/resolvent.jl:146-252    _complement_solve: X[:, j] solves Q (H - s_j) Q x = Q B[:, j], x
                              orthogonal to the basis, Q = 1 - basis basis', by a conjugate gradient
                              on all columns in lockstep, each with its own scalars, preconditioned by
                              1 / hypot(D - s_j, eta); per-column targets tol ||Q B_j||, columns
                              converged from the start (x_j = 0), the round-off floor (true residuals
                              checked once the recurrence residual is below the cap), the positivity
                              check, and the final true-residual acceptance

`H` is any operator with `matvec` on column blocks (the oracle's KronFreeOperator or CApply).
"""
from __future__ import annotations

import numpy as np

EPS = np.finfo(np.float64).eps
FLOOR_CAP = 1000          # src/resolvent.jl:115
FLOOR_PATIENCE = 5        # src/resolvent.jl:117


class ComplementError(RuntimeError):
    pass


def _colnorms(A):
    return np.sqrt(np.sum(np.abs(A) ** 2, axis=0))


def _colredot(A, B):
    """src/resolvent.jl:111."""
    return np.real(np.sum(np.conj(A) * B, axis=0))


def complement_solve(H, D, basis, B, shifts, tol, maxiter, eta=0.01, scale=None):
    """src/resolvent.jl:146-252.  Returns (X, iterations, residuals, from_start, at_floor,
    floor_residuals) with 0-based column indices."""
    B = np.asarray(B, dtype=np.float64)
    n = B.shape[1]
    shifts = np.asarray(shifts, dtype=np.float64)
    if len(shifts) != n:
        raise ValueError(f"{n} columns and {len(shifts)} shifts")
    scale = _colnorms(B) if scale is None else np.asarray(scale, dtype=np.float64)
    if len(scale) != n:
        raise ValueError(f"{n} columns and {len(scale)} scales")
    basis = np.asarray(basis, dtype=np.float64)

    def project(Y):
        if basis.shape[1] == 0:
            return Y
        return Y - basis @ (basis.T @ Y)

    S = shifts[None, :]
    Minv = 1.0 / np.hypot(np.asarray(D, dtype=np.float64)[:, None] - S, eta)
    cap = FLOOR_CAP * EPS * scale
    QB = project(B.copy())
    b = _colnorms(QB)
    goal = tol * b
    from_start = [j for j in range(n) if b[j] <= cap[j]]
    met = np.zeros(n, dtype=bool)
    atfloor = np.zeros(n, dtype=bool)
    atfloor[from_start] = True
    QB = QB * (~atfloor)[None, :]
    X = np.zeros_like(B)
    Rr = QB.copy()
    Z = project(Minv * Rr)
    P = Z.copy()
    rho = _colredot(Rr, Z)

    def true_residuals():
        T = H.matvec(np.asfortranarray(X)) - X * S
        T = project(T) - QB
        return _colnorms(T)

    rn = b.copy()
    anchor = np.full(n, np.inf)
    stalled = np.zeros(n, dtype=int)
    done = lambda: bool(np.all(met | atfloor))
    iterations = 0
    while not done() and iterations < maxiter:
        iterations += 1
        AP = H.matvec(np.asfortranarray(P)) - P * S
        AP = project(AP)
        kappa = _colredot(P, AP)
        for j in range(n):
            if met[j] or atfloor[j] or kappa[j] > 0:
                continue
            if rn[j] <= cap[j]:
                atfloor[j] = True
                continue
            raise ComplementError(
                f"the linear solve on the complement is not positive on the complement at column {j + 1} "
                f"(<p, (H - s) p> = {kappa[j]} after {iterations} iterations)")
        active = ~(met | atfloor)
        alpha = np.where(active, rho / np.where(active, kappa, 1.0), 0.0)
        X = X + P * alpha[None, :]
        Rr = Rr - AP * alpha[None, :]
        rn = _colnorms(Rr)
        met |= active & (rn <= goal)
        near = ~(met | atfloor) & (rn <= cap)
        if near.any():
            tr = true_residuals()
            for j in np.nonzero(near)[0]:
                if tr[j] < anchor[j] / 2:
                    anchor[j], stalled[j] = tr[j], 0
                else:
                    stalled[j] += 1
                if stalled[j] >= FLOOR_PATIENCE and tr[j] <= cap[j]:
                    atfloor[j] = True
        if done():
            break
        Z = project(Minv * Rr)
        rho_n = _colredot(Rr, Z)
        beta = np.where(met | atfloor, 0.0, rho_n / np.where(met | atfloor, 1.0, rho))
        P = Z + P * beta[None, :]
        rho = rho_n
    tr = true_residuals()
    for j in range(n):
        if not (met[j] or atfloor[j]) and tr[j] <= cap[j]:
            atfloor[j] = True
    if not done():
        j = int(np.nonzero(~(met | atfloor))[0][0])
        raise ComplementError(f"the linear solve on the complement did not converge at column {j + 1}: residual "
                              f"{rn[j] / b[j]} after {iterations} iterations (tolerance {tol}, at most {maxiter})")
    met0 = met.copy()
    for j in range(n):
        if j in from_start:
            continue
        if met[j] and tr[j] > 10 * goal[j]:
            met[j] = False
            atfloor[j] = True
        if atfloor[j] and tr[j] > cap[j]:
            raise ComplementError(f"the linear solve on the complement did not converge at column {j + 1} "
                                  f"({'met its tolerance by the recurrence' if met0[j] else 'at the floor'}, "
                                  f"true residual {tr[j] / scale[j]})")
    residuals = np.array([tr[j] / b[j] if met[j] else 0.0 for j in range(n)])
    at_floor = [j for j in range(n) if atfloor[j] and j not in from_start]
    floor_residuals = np.array([tr[j] / scale[j] if j in at_floor else 0.0 for j in range(n)])
    return X, iterations, residuals, from_start, at_floor, floor_residuals
