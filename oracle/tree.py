"""A two-level materialization for the golden checks (test infrastructure only).

Restates the parts of src/materialize.jl the pinned goldens exercise:
  - a leaf takes every term whose modes all lie in it (routing, src/tree.jl:500-529);
  - a branch axis per child holds the child's kept basis: its kept energies as a diagonal
    factor, and each routed term's factors on that child as the port V' (⊗ O) V in the kept
    basis (src/materialize.jl:583-603, 822-914);
  - the constant constant + 4 n_g' E_C n_g is added at the root only
    (test/test_materialize.jl:121-124 states this);
  - Dense is LAPACK on Matrix(H) (src/solvers.jl:44-50).
Arithmetic here is complex throughout; for a real-by-structure node the imaginary parts vanish
and the energies equal the real path's (src/character.jl:249).
"""
from __future__ import annotations

import numpy as np

from . import kfref


def dense_solve(H, m):
    """solve(::Dense, H, m) (src/solvers.jl:44-50): the lowest m pairs of Matrix(H)."""
    M = H.to_matrix()
    M = (M + M.conj().T) / 2
    w, V = np.linalg.eigh(M)
    if 0 < m < len(w):
        return w[:m], V[:, :m]
    return w, V


def materialize_leaf(spec, theta, bases, keep, root=False, ports=()):
    """A leaf node: all terms on its modes, Dense, the lowest `keep` states.

    Returns dict(energies, vectors, ports={(mode, kind): kept-basis matrix}, H).
    """
    terms = kfref.leaf_terms(spec, theta, bases)
    const = kfref.constant_term(spec, theta) if root else 0.0
    H = kfref.KronFreeOperator([b.dim for b in bases.values()], terms, constant=const)
    E, V = dense_solve(H, keep)
    out = {"energies": E, "vectors": V, "H": H, "bases": bases, "ports": {}}
    names = list(bases.keys())
    for mode, kind in ports:
        op = kfref.localop(bases[mode], kind)
        full = kfref.apply_axis(op, V.reshape(-1, order="F").astype(np.complex128),
                                [b.dim for b in bases.values()] + [V.shape[1]], names.index(mode))
        out["ports"][(mode, kind)] = V.conj().T @ full.reshape(V.shape, order="F")
    return out


def _kept_port(child, factors):
    """V' (⊗_f O_f) V for the factors (mode, kind, k) that lie in `child` (a joint port if several)."""
    bases = child["bases"]
    names = list(bases.keys())
    dims = [b.dim for b in bases.values()]
    V = child["vectors"]
    Y = V.reshape(-1, order="F").astype(np.complex128)
    for mode, kind, k in sorted(factors, key=lambda f: names.index(f[0])):
        Y = kfref.apply_axis(kfref.localop(bases[mode], kind, k), Y, dims + [V.shape[1]], names.index(mode))
    return V.conj().T @ Y.reshape(V.shape, order="F")


def materialize_branch(spec, theta, leaves, keeps, top_keep):
    """A root over leaf children: each leaf solved by Dense keeping `keeps[i]`, the root by Dense.

    `leaves` is a list of {mode: basis} dicts.  Returns dict(energies, vectors, children, H).
    """
    children = [materialize_leaf(spec, theta, b, k) for b, k in zip(leaves, keeps)]
    mode_child = {m: i for i, b in enumerate(leaves) for m in b}
    terms = []
    for c, fs in kfref.circuit_terms(spec, theta):
        owners = sorted({mode_child[m] for m, _, _ in fs})
        if len(owners) <= 1:
            continue                                   # routed to a leaf
        factors = []
        for a in owners:
            P = _kept_port(children[a], [f for f in fs if mode_child[f[0]] == a])
            factors.append((a, kfref.DenseOp(P)))
        terms.append((c, factors))
    for a, ch in enumerate(children):
        terms.append((1.0, [(a, kfref.DiagonalOp(ch["energies"]))]))
    dims = [len(ch["energies"]) for ch in children]
    H = kfref.KronFreeOperator(dims, terms, constant=kfref.constant_term(spec, theta))
    E, V = dense_solve(H, top_keep)
    return {"energies": E, "vectors": V, "children": children, "H": H}
