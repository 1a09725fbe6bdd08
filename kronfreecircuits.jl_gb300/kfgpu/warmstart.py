"""The learned warm start: an MLP maps a node's circuit parameters theta to its initial LOBPCG block.

Pipeline (all GPU work through libkfgpu):
  1. label: the plain solver's own eigenvectors V(theta) (N x m) for sampled theta;
  2. POD: the leading `k` left singular vectors of all labels stacked (a randomized range finder
     with two power iterations, host NumPy -- offline data preparation of the caller's side);
  3. targets: C(theta) = POD' V(theta) (k x m), each column's sign fixed so that its largest
     entry is positive (eigenvectors are defined up to sign);
  4. train the din -> 256 -> 256 -> k m network with the library's own forward / backward / Adam
     kernels (kfgpu.mlp);
  5. warm start: X0 = POD C_pred(theta), handed to kf_solve as the warm-start block, with the
     solver's check: if the largest residual after `fallback_iters` iterations exceeds
     `fallback_resid`, the solve restarts from a random block (the plain method remains the
     fallback and the reference).

The reference's warm start is the previous solution's vectors (src/materialize.jl:656-670,
`_initial_block`); this is the learned extension of that hook for parameter sweeps.
"""
from __future__ import annotations

import time

import numpy as np

from . import circuits
from .mlp import MLP
from .operator import KronFreeOperator
from .solvers import LOBPCG, solve

# The two-transmon circuit's parameter box for the learned warm start: a +-33% box around the
# reference fixture's theta (E_J1 = 30, E_C1 = 1.2, n_g1 = 0.25, E_J2 = 25, E_C2 = 1.0, n_g2 = 0,
# g = 0.3), offset charges over half a period.
THETA_RANGES = {"E_J1": (20.0, 40.0), "E_C1": (0.8, 1.6), "n_g1": (0.0, 0.5), "E_J2": (17.0, 33.0),
                "E_C2": (0.67, 1.33), "n_g2": (0.0, 0.5), "g": (0.2, 0.4)}
KEYS = list(THETA_RANGES)


def sample_thetas(n, seed):
    rng = np.random.default_rng(seed)
    return [{k: rng.uniform(*THETA_RANGES[k]) for k in KEYS} for _ in range(n)]


def theta_matrix(thetas):
    return np.array([[t[k] for k in KEYS] for t in thetas], dtype=np.float32)


def operator(theta, ncut=30):
    dims, terms, const = circuits.two_transmon_flat(theta, ncut)
    return KronFreeOperator(dims, terms, constant=const)


def tolerance(H):
    return 1e-8 * H.gershgorin_bound()


def label(thetas, m=12, ncut=30, preconditioner="separable"):
    """The solver's eigenvectors (N x m) and energies for each theta (FP64 LOBPCG, product seed)."""
    Vs, Es = [], []
    for th in thetas:
        H = operator(th, ncut)
        E, V, _ = solve(LOBPCG(tol=tolerance(H), preconditioner=preconditioner), H, m)
        Vs.append(V)
        Es.append(E)
        H.close()
    return Vs, Es


def pod_basis(Vs, k=128, seed=0):
    """Leading k left singular vectors of [V_1 ... V_n] (randomized range finder, 2 power steps)."""
    A = np.concatenate(Vs, axis=1)
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(A @ rng.standard_normal((A.shape[1], k + 32)))
    for _ in range(2):
        Q, _ = np.linalg.qr(A @ (A.T @ Q))
    U, s, _ = np.linalg.svd(Q.T @ A, full_matrices=False)
    return np.ascontiguousarray(Q @ U[:, :k])


def targets(Vs, POD):
    """C = POD' V per theta, sign-fixed per column, flattened column-major (k*m values)."""
    out = []
    for V in Vs:
        C = POD.T @ V
        idx = np.argmax(np.abs(C), axis=0)
        C = C * np.sign(C[idx, np.arange(C.shape[1])])[None, :]
        out.append(C.reshape(-1, order="F"))
    return np.array(out, dtype=np.float32)


class WarmStart:
    """A trained network plus its POD basis: `block(theta)` is the N x m warm-start block."""

    def __init__(self, POD, m, hidden=256, seed=0):
        self.POD, self.m = POD, m
        self.net = MLP(len(KEYS), hidden, POD.shape[1] * m, seed=seed)

    def fit(self, thetas, Y, epochs=200, batch=256, lr=1e-3, seed=0):
        X = theta_matrix(thetas)
        self.net.fit_scaling(X, Y)
        return self.net.train(X, Y, epochs=epochs, batch=batch, lr=lr, seed=seed)

    def blocks(self, thetas):
        C = self.net.forward(theta_matrix(thetas)).astype(np.float64)
        k = self.POD.shape[1]
        return [self.POD @ c.reshape(k, self.m, order="F") for c in C]


def evaluate(ws, thetas, m=12, ncut=30, fallback_resid=1e-2, fallback_iters=3, preconditioner="separable",
             product_arm=False):
    """LOBPCG iterations and wall time per theta: warm-started by the network vs a random start and,
    with `product_arm`, vs the solver's default start without the network (the product seed,
    src/lobpcg.jl:247), all with the same preconditioner."""
    X0s = ws.blocks(thetas) if ws is not None else [None] * len(thetas)
    rows = []
    for th, X0 in zip(thetas, X0s):
        H = operator(th, ncut)
        tol = tolerance(H)
        t0 = time.perf_counter()
        Er, _, sr = solve(LOBPCG(tol=tol, seed="random", preconditioner=preconditioner), H, m)
        tr = time.perf_counter() - t0
        row = {"random_iters": sr["iterations"], "random_s": tr, "E": Er}
        if product_arm:
            t0 = time.perf_counter()
            Ep, _, sp = solve(LOBPCG(tol=tol, seed="product", preconditioner=preconditioner), H, m)
            row.update({"product_iters": sp["iterations"], "product_s": time.perf_counter() - t0, "E_product": Ep})
        if X0 is not None:
            t0 = time.perf_counter()
            # guards from the product seed, as the reference's warm starts take them (src/lobpcg.jl:182-190)
            Ew, _, sw = solve(LOBPCG(tol=tol, seed="product", preconditioner=preconditioner,
                                     fallback_iters=fallback_iters, fallback_resid=fallback_resid), H, m, X0=X0)
            tw = time.perf_counter() - t0
            row.update({"warm_iters": sw["iterations"], "warm_s": tw, "fell_back": sw["fell_back"],
                        "max_dE": float(np.max(np.abs(Ew - Er))), "E_warm": Ew})
        rows.append(row)
        H.close()
    return rows
