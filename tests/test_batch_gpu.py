"""Batched leaf solves (kf_batch_solve) against the oracle: fluxonium leaves of uneven sizes
(the batched sweep's leaves, 5-point stencil on [-5 pi, 5 pi]), the lowest 10 pairs each; every
eigenvalue within 1e-9 relative of LAPACK on the oracle's matrix and every residual, recomputed
by the oracle's operator, below max(tol, 10 eps ||H||).  Then a two-leaf chain coupled by
g n_1 n_2 (the imaginary grid n ports become -g I_1 (x) I_2 in the real expansion), its parent
built from the batched leaves' vectors and solved, against a dense solve of the same parent."""
import numpy as np
import pytest

from oracle import circuits as ocirc
from oracle import solvers as osol

pytestmark = pytest.mark.gpu


def _leaves(k, seed):
    from kfgpu import circuits
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(k):
        th = circuits.fluxonium_theta(rng)
        n = int(rng.integers(200, 601))
        dims, terms = circuits.fluxonium_leaf(th, n)
        out.append((th, n, dims, terms))
    return out


def test_batched_leaves_match_dense(cuda):
    from kfgpu.batch import autotune, batch_solve
    leaves = _leaves(16, 3)
    ops = [(dims, terms, 0.0) for _, _, dims, terms in leaves]
    tol = 1e-9
    tile = autotune(ops, [10] * len(ops), tol)
    assert tile in (128, 256, 512)
    Es, Vs, iters, resid = batch_solve(ops, [10] * len(ops), tol)
    for (th, n, _, _), E, V in zip(leaves, Es, Vs):
        Ho = ocirc.fluxonium_operator(th, n)
        Eref, _ = osol.dense_solve(Ho, 10)
        assert np.max(np.abs(E - Eref) / np.maximum(np.abs(Eref), 1.0)) < 1e-9
        R = Ho.matvec(V) - V * E[None, :]
        thr = max(tol, 10 * np.finfo(float).eps * Ho.gershgorin_bound())
        assert np.max(np.sqrt(np.sum(R ** 2, axis=0))) <= thr * 1.0001
        assert np.linalg.norm(V.T @ V - np.eye(10)) < 1e-9


def test_batched_chain_parent(cuda):
    from kfgpu import KronFreeOperator, LOBPCG, solve, ops as P
    from kfgpu.batch import batch_solve
    from kfgpu.ops import PhaseGrid, localop
    leaves = _leaves(2, 8)
    ops = [(dims, terms, 0.0) for _, _, dims, terms in leaves]
    Es, Vs, _, _ = batch_solve(ops, [10, 10], 1e-9)
    g = 0.05
    ports = []
    for (th, n, _, _), V in zip(leaves, Vs):
        A = localop(PhaseGrid(-5 * np.pi, 5 * np.pi, n, 4), "n", part="im").dense()   # n = i A
        ports.append(V.T @ A @ V)
    terms = [(1.0, [(0, P.DiagonalOp(Es[0]))]), (1.0, [(1, P.DiagonalOp(Es[1]))]),
             (-g, [(0, P.DenseOp(ports[0])), (1, P.DenseOp(ports[1]))])]
    H = KronFreeOperator([10, 10], terms, block_capacity=24)
    E, V, _ = solve(LOBPCG(tol=1e-9), H, 20)
    M = np.kron(np.eye(10), np.diag(Es[0])) + np.kron(np.diag(Es[1]), np.eye(10)) - g * np.kron(ports[1], ports[0])
    assert np.max(np.abs(E - np.linalg.eigvalsh(M)[:20])) < 1e-9
