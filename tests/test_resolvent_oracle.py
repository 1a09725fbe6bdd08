"""The oracle's restatement of the linear solve on the complement of known states
(src/resolvent.jl:146-252, oracle/resolvent.py) pinned against an independent computation: the
exact solution x_j = sum over the complement's eigenpairs (E_c, v_c) of v_c <v_c, b_j> / (E_c - s_j)
from a dense eigendecomposition.  Sternheimer shifts (the known states' own energies) keep
H - s_j positive on the complement, as in the reference's use.  Also: a right-hand side inside the
known span is converged from the start with x = 0, a shift above the complement's lowest energy is
"not positive on the complement", and too few iterations "did not converge".
"""
import numpy as np
import pytest

from oracle import kfref, resolvent as ores, solvers as osol


def _oracle_op(dims, terms):
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
    return kfref.KronFreeOperator(dims, conv)


def _cases():
    from kfgpu import circuits
    rng = np.random.default_rng(7)
    th = circuits.fluxonium_theta(rng)
    yield "fluxonium 301", _oracle_op(*circuits.fluxonium_leaf(th, 301)), 6
    dims, terms = circuits.three_mode_leaf(circuits.three_mode_theta(rng), ncut=4, n2=16, n3=10)
    yield "three-mode 1440", _oracle_op(dims, terms), 8


@pytest.mark.parametrize("case", [0, 1])
def test_complement_solve_matches_dense(case):
    name, H, nb = list(_cases())[case]
    M = H.to_matrix().real
    E, V = np.linalg.eigh((M + M.T) / 2)
    basis, Eb = V[:, :nb], E[:nb]
    rng = np.random.default_rng(11 + case)
    B = rng.standard_normal((H.N, nb))
    B[:, 2] = basis @ rng.standard_normal(nb)            # inside the known span: converged from the start
    X, it, res, fs, af, fres = ores.complement_solve(H, H.diagonal().real, basis, B, Eb, tol=1e-10, maxiter=2000)
    Vc, Ec = V[:, nb:], E[nb:]
    Xd = Vc @ ((Vc.T @ B) / (Ec[:, None] - Eb[None, :]))
    scale = np.max(np.abs(Xd), axis=0)
    for j in range(nb):
        if j == 2:
            continue
        assert np.max(np.abs(X[:, j] - Xd[:, j])) < 1e-7 * scale[j], (name, j)
    assert fs == [2] and np.all(X[:, 2] == 0)
    assert np.max(np.abs(basis.T @ X)) < 1e-10 * np.max(np.abs(X))
    assert it > 1 and np.all(res[[j for j in range(nb) if j != 2]] <= 10 * 1e-10)


def test_complement_solve_errors():
    name, H, nb = list(_cases())[0]
    M = H.to_matrix().real
    E, V = np.linalg.eigh((M + M.T) / 2)
    basis = V[:, :nb]
    B = np.random.default_rng(3).standard_normal((H.N, 2))
    # a shift above the complement's lowest energy: H - s is not positive there
    with pytest.raises(ores.ComplementError, match="not positive on the complement"):
        ores.complement_solve(H, H.diagonal().real, basis, B, [E[0], E[nb] + 0.5 * (E[nb + 1] - E[nb])],
                              tol=1e-10, maxiter=2000)
    with pytest.raises(ores.ComplementError, match="did not converge"):
        ores.complement_solve(H, H.diagonal().real, basis, B, E[:2], tol=1e-12, maxiter=3)
    with pytest.raises(ValueError, match="shifts"):
        ores.complement_solve(H, H.diagonal().real, basis, B, E[:3], tol=1e-10, maxiter=10)
