"""The GPU linear solve on the complement of known states (kf_complement_solve, src/resolvent.jl:
146-252) against the exact solution from a dense eigendecomposition of the complement and against
the oracle's restatement (oracle/resolvent.py: the same column states, iteration counts within 3),
on a fluxonium leaf, a small three-mode leaf and the two-transmon flat space; at the three-mode
leaf's full size (N = 671,744) through the true residual recomputed by the oracle's own apply and
the orthogonality to the basis; and the reference's errors.
"""
import numpy as np
import pytest

from oracle import capply, kfref, resolvent as ores

pytestmark = pytest.mark.gpu


def _oracle_op(dims, terms, constant=0.0):
    from kfgpu import ops as P
    conv = []
    for c, fs in terms:
        g = []
        for a, op in fs:
            if isinstance(op, P.DiagonalOp):
                g.append((a, kfref.DiagonalOp(op.d)))
            elif isinstance(op, P.ShiftOp):
                g.append((a, kfref.ShiftOp(op.n, op.s, op.factor)))
            elif isinstance(op, P.BandedOp):
                g.append((a, kfref.BandedOp(op.n, op.offsets, op.weights)))
            else:
                g.append((a, kfref.DenseOp(op.dense())))
        conv.append((c, g))
    return kfref.KronFreeOperator(dims, conv, constant=constant)


def _case(i):
    from kfgpu import KronFreeOperator, circuits
    from kfgpu import warmstart as W
    rng = np.random.default_rng(7)
    if i == 0:
        dims, terms = circuits.fluxonium_leaf(circuits.fluxonium_theta(rng), 301)
        const, nb = 0.0, 6
    elif i == 1:
        dims, terms = circuits.three_mode_leaf(circuits.three_mode_theta(rng), ncut=4, n2=16, n3=10)
        const, nb = 0.0, 8
    else:
        dims, terms, const = circuits.two_transmon_flat(W.sample_thetas(1, seed=5)[0])
        nb = 12
    return KronFreeOperator(dims, terms, constant=const), _oracle_op(dims, terms, const), nb


@pytest.mark.parametrize("case", [0, 1, 2])
def test_complement_solve_matches_dense_and_oracle(cuda, case):
    from kfgpu.resolvent import complement_solve
    H, Ho, nb = _case(case)
    M = Ho.to_matrix().real
    E, V = np.linalg.eigh((M + M.T) / 2)
    basis, Eb = V[:, :nb], E[:nb]
    rng = np.random.default_rng(11 + case)
    B = rng.standard_normal((H.N, nb))
    B[:, 2] = basis @ rng.standard_normal(nb)             # inside the known span: x = 0 from the start
    X, it, res, fs, af, fres = complement_solve(H, basis, B, Eb, tol=1e-10, maxiter=2000)
    Vc, Ec = V[:, nb:], E[nb:]
    Xd = Vc @ ((Vc.T @ B) / (Ec[:, None] - Eb[None, :]))
    for j in range(nb):
        if j != 2:
            assert np.max(np.abs(X[:, j] - Xd[:, j])) < 1e-7 * np.max(np.abs(Xd[:, j])), j
    assert fs == [2] and np.all(X[:, 2] == 0)
    assert all(res[j] <= 10 * 1e-10 for j in range(nb) if j != 2)
    Xo, ito, reso, fso, afo, _ = ores.complement_solve(Ho, Ho.diagonal().real, basis, B, Eb, tol=1e-10, maxiter=2000)
    assert fso == fs and afo == af and abs(ito - it) <= 3, (it, ito)
    H.close()


def test_complement_solve_full_size(cuda):
    """N = 671,744: the basis is the FP64 LOBPCG solve's 12 lowest states; the shifts stay below the
    lowest energy, so H - s is positive on the whole space."""
    from kfgpu import KronFreeOperator, LOBPCG, circuits, solve
    from kfgpu.resolvent import complement_solve
    th = circuits.three_mode_theta(np.random.default_rng(20261205))
    dims, terms = circuits.three_mode_leaf(th)
    H = KronFreeOperator(dims, terms)
    E, V, _ = solve(LOBPCG(tol=1e-9 * H.gershgorin_bound(), precision="mixed", preconditioner="separable"), H, 12)
    rng = np.random.default_rng(3)
    B = rng.standard_normal((H.N, 6))
    shifts = E[0] - np.array([0.0, 0.1, 0.5, 1.0, 2.0, 5.0])
    X, it, res, fs, af, fres = complement_solve(H, V, B, shifts, tol=1e-9, maxiter=5000)
    assert fs == [] and it > 1
    Ho = capply.CApply(_oracle_op(dims, terms))
    QB = B - V @ (V.T @ B)
    T = Ho.matvec(np.asfortranarray(X)) - X * shifts[None, :]
    T = T - V @ (V.T @ T) - QB
    rel = np.sqrt(np.sum(T ** 2, axis=0)) / np.sqrt(np.sum(QB ** 2, axis=0))
    assert np.all(rel <= 1e-8), rel
    assert np.max(np.abs(V.T @ X)) < 1e-9 * np.max(np.abs(X))
    H.close()


def test_complement_solve_errors(cuda):
    from kfgpu import ConvergenceError, DimensionMismatch
    from kfgpu.resolvent import complement_solve
    H, Ho, nb = _case(0)
    M = Ho.to_matrix().real
    E, V = np.linalg.eigh((M + M.T) / 2)
    basis = V[:, :nb]
    B = np.random.default_rng(3).standard_normal((H.N, 2))
    with pytest.raises(ConvergenceError, match="not positive on the complement"):
        complement_solve(H, basis, B, [E[0], E[nb] + 0.5 * (E[nb + 1] - E[nb])], tol=1e-10, maxiter=2000)
    with pytest.raises(ConvergenceError, match="did not converge"):
        complement_solve(H, basis, B, E[:2], tol=1e-12, maxiter=3)
    with pytest.raises(DimensionMismatch, match="shifts"):
        complement_solve(H, basis, B, E[:3], tol=1e-10, maxiter=10)
    H.close()
