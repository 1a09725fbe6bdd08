"""The device Rayleigh-Ritz eigensolver of the FP32 LOBPCG phase (kf_rr.cu: FP32 Jacobi on one CTA)
against numpy.linalg.eigh of the same symmetric matrix assembled from the Gram blocks the way the
host path assembles it (upper triangle of the merged [X_a Q]'[HX_a HZ] layout, or the packed
[X_a'HX_a | X_a'HZ | Q'HZ] blocks), odd and even sizes up to 64 with clustered eigenvalues: Ritz
values within 2e-6 ||A||, the coefficient layout [C_x | [0; C_z]], the retained eigenvectors
orthonormal to 1e-5 and spanning the same invariant subspace; and the failed-Cholesky path (X kept,
P dropped, theta untouched).  FP32 is the phase's own precision: it stops at 1e-6 ||H||.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(G, ldg, packed, na, k, status=0):
    from kfgpu import _abi
    ns = na + k
    Cm = np.zeros(ns * 2 * na)
    th = np.full(na, 7.0)
    Gc = np.ascontiguousarray(G, dtype=np.float64)
    _abi.check(_abi.lib().kf_test_rr_eig(Gc.ctypes.data, ldg, packed, na, k, status, Cm.ctypes.data, th.ctypes.data))
    return Cm.reshape(2 * na, ns).T, th


def _sym(ns, rng, cluster=False):
    Q, _ = np.linalg.qr(rng.standard_normal((ns, ns)))
    ev = np.sort(rng.uniform(-20, 2000, ns))
    if cluster:
        ev[:6] = -18.0 + np.array([0, 3e-11, 1e-9, 0.5, 0.5 + 1e-8, 1.0])
    return (Q * ev) @ Q.T


@pytest.mark.parametrize("na,k", [(18, 36), (12, 24), (5, 0), (17, 30), (20, 44), (1, 1), (9, 10)])
@pytest.mark.parametrize("packed", [0, 1])
def test_rr_device_matches_eigh(cuda, na, k, packed):
    rng = np.random.default_rng(na * 100 + k + packed)
    ns = na + k
    A = _sym(ns, rng, cluster=ns >= 8)
    if packed:
        G = np.concatenate([A[:na, :na].ravel(order="F"), A[:na, na:].ravel(order="F"), A[na:, na:].ravel(order="F")])
        ldg = ns
    else:
        ldg = ns
        # the kernel reads the upper triangle only: a lower triangle of garbage must not matter
        G = (np.triu(A) + np.tril(np.full((ns, ns), 123.0), -1)).ravel(order="F")
    Cm, th = _run(G, ldg, packed, na, k)
    w, V = np.linalg.eigh(A)
    nrm = np.max(np.abs(w))
    assert np.max(np.abs(th - w[:na])) < 2e-6 * nrm, np.abs(th - w[:na])
    Cx, Cp = Cm[:, :na], Cm[:, na:]
    assert np.all(Cp[:na, :] == 0) and np.allclose(Cp[na:, :], Cx[na:, :])
    assert np.max(np.abs(Cx.T @ Cx - np.eye(na))) < 1e-5
    # the retained vectors span the eigenvectors of the na lowest eigenvalues (up to the cluster
    # above the cut, when there is one)
    gap = w[na] - w[na - 1] if na < ns else np.inf
    if gap > 1e-3 * nrm:
        P = V[:, :na] @ V[:, :na].T
        bound = max(20 * 6e-8 * np.linalg.norm(A) / gap, 1e-5)     # FP32: eps ||A|| / gap
        assert np.max(np.abs(P @ Cx - Cx)) < bound
    # residuals ||A c - theta c|| relative to ||A||
    R = A @ Cx - Cx * th[None, :]
    assert np.max(np.linalg.norm(R, axis=0)) < 2e-5 * nrm


def test_rr_device_failed_cholesky_keeps_x(cuda):
    na, k = 6, 10
    A = _sym(na + k, np.random.default_rng(1))
    Cm, th = _run(A.ravel(order="F"), na + k, 0, na, k, status=1)
    assert np.array_equal(Cm[:, :na], np.eye(na + k)[:, :na]) and np.all(Cm[:, na:] == 0)
    assert np.all(th == 7.0)


def test_solve_through_device_rr_matches_dense(cuda, monkeypatch):
    """A mixed-precision LOBPCG solve with the device Rayleigh-Ritz (KF_DEVICE_RR=1, read per solve)
    on the two-transmon flat space reaches the oracle's Dense eigenvalues as the default path does."""
    from kfgpu import LOBPCG, circuits, solve
    from kfgpu import warmstart as W
    from oracle import kfref, solvers as osol
    th = W.sample_thetas(1, seed=9)[0]
    H = W.operator(th)
    dims, terms, const = circuits.two_transmon_flat(th)
    from kfgpu import ops as P
    conv = []
    for c, fs in terms:
        conv.append((c, [(a, kfref.DiagonalOp(op.d) if isinstance(op, P.DiagonalOp) else
                          kfref.ShiftOp(op.n, op.s, op.factor)) for a, op in fs]))
    Ed, _ = osol.dense_solve(kfref.KronFreeOperator(dims, conv, constant=const), 12)
    tol = W.tolerance(H)
    monkeypatch.setenv("KF_DEVICE_RR", "1")
    E1, _, st1 = solve(LOBPCG(tol=tol, precision="mixed", preconditioner="separable"), H, 12)
    monkeypatch.delenv("KF_DEVICE_RR")
    E0, _, st0 = solve(LOBPCG(tol=tol, precision="mixed", preconditioner="separable"), H, 12)
    for E in (E0, E1):
        assert np.max(np.abs(E - Ed) / np.maximum(1.0, np.abs(Ed))) < 1e-9
    H.close()
