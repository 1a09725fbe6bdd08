"""The synthetic circuits of the measured workloads, built the reference's way (test infrastructure only).

Each circuit is written as a kronfree-spec dictionary (the reference's input format, src/spec.jl)
and expanded by `kfref.circuit_terms` + the real expansion, i.e. the route
materialize -> _real_node_terms -> KronFreeOperator takes in the reference
(src/materialize.jl:583-647).  The GPU side builds the same Hamiltonians from its own port
operators; tests compare the two.
"""
from __future__ import annotations

import numpy as np

from . import kfref

PI = np.pi


def three_mode_spec():
    """H = 4E_C1 n1^2 - E_C2 d2^2 - E_C3 d3^2 + E_L/2 (phi2^2 + phi3^2) - 2E_J cos phi1 cos phi2 - E_J' cos(phi2 - phi3).

    -E_C d^2 is `n2port` with coefficient E_C, i.e. a spec diagonal E_C/4; -2E_J cos phi1 cos phi2 is
    the pair of cosines E_J (phi1 + phi2) and E_J (phi1 - phi2).
    """
    return {
        "format": "kronfree-spec", "version": 1,
        "parameters": ["E_J", "E_C1", "E_C2", "E_C3", "E_L", "E_Jp"],
        "modes": [{"name": "phi1", "type": "c"}, {"name": "phi2", "type": "e"}, {"name": "phi3", "type": "e"}],
        "E_C": [["E_C1", "0", "0"], ["0", "E_C2/4", "0"], ["0", "0", "E_C3/4"]],
        "E_L": [["0", "0", "0"], ["0", "E_L", "0"], ["0", "0", "E_L"]],
        "flux_linear": ["0", "0", "0"],
        "n_g": ["0", "0", "0"],
        "cosines": [
            {"energy": "E_J", "omega": [1, 1, 0], "offset": "0"},
            {"energy": "E_J", "omega": [1, -1, 0], "offset": "0"},
            {"energy": "E_Jp", "omega": [0, 1, -1], "offset": "0"},
        ],
    }


def three_mode_theta(rng):
    """theta ~ the uniform ranges of the three-mode leaf workload."""
    return {"E_J": rng.uniform(5, 15), "E_C1": rng.uniform(0.02, 0.1), "E_C2": rng.uniform(0.5, 2),
            "E_C3": rng.uniform(0.5, 2), "E_L": rng.uniform(0.02, 0.2), "E_Jp": rng.uniform(0.5, 2)}


def three_mode_operator(theta, ncut=20, n2=256, n3=64):
    bases = {"phi1": kfref.ChargeBasis(ncut), "phi2": kfref.PhaseGrid(-4 * PI, 4 * PI, n2, 4),
             "phi3": kfref.PhaseGrid(-3 * PI, 3 * PI, n3, 4)}
    terms = kfref.leaf_terms(three_mode_spec(), theta, bases, real=True)
    return kfref.KronFreeOperator([b.dim for b in bases.values()], _merge(terms))


def fluxonium_theta(rng):
    """theta ~ U: E_J [3,10], E_C [0.5,1.5], E_L [0.2,1.2], phi_ext [0, 2 pi]."""
    return {"E_J": rng.uniform(3, 10), "E_C": rng.uniform(0.5, 1.5), "E_L": rng.uniform(0.2, 1.2),
            "phi_ext": rng.uniform(0, 2 * PI)}


def fluxonium_spec():
    """-E_C d^2 (5-point) + E_L/2 phi^2 - E_J cos(phi - phi_ext): E_C/4 on the spec diagonal."""
    return {
        "format": "kronfree-spec", "version": 1,
        "parameters": ["E_J", "E_C", "E_L", "phi_ext"],
        "modes": [{"name": "phi", "type": "e"}],
        "E_C": [["E_C/4"]], "E_L": [["E_L"]], "flux_linear": ["0"], "n_g": ["0"],
        "cosines": [{"energy": "E_J", "omega": [1], "offset": "-phi_ext"}],
    }


def fluxonium_operator(theta, npts):
    bases = {"phi": kfref.PhaseGrid(-5 * PI, 5 * PI, npts, 4)}
    terms = kfref.leaf_terms(fluxonium_spec(), theta, bases, real=True)
    return kfref.KronFreeOperator([npts], _merge(terms))


def _same_op(a, b):
    if type(a) is not type(b) or a.n != b.n:
        return False
    if isinstance(a, kfref.ShiftOp):
        return a.s == b.s and a.factor == b.factor
    if isinstance(a, kfref.BandedOp):
        return a.offsets == b.offsets and all(np.array_equal(x, y) for x, y in zip(a.weights, b.weights))
    if isinstance(a, kfref.DiagonalOp):
        return np.array_equal(a.d, b.d)
    return np.array_equal(a.M, b.M)


def _merge(terms):
    """Sum real terms on equal factors, as the reference's `_real_node_terms` sums equal keys
    (src/materialize.jl:616-647); terms whose coefficients cancel are dropped."""
    out = []
    for c, fs in terms:
        for k, (c2, fs2) in enumerate(out):
            if len(fs) == len(fs2) and all(a == a2 and _same_op(o, o2) for (a, o), (a2, o2) in zip(fs, fs2)):
                out[k] = (c2 + c, fs2)
                break
        else:
            out.append((c, fs))
    return [(c, fs) for c, fs in out if c != 0]


def dense_parent_operator(rng, d=48):
    """The parent-level dense contraction workload: three children keeping d states each,
    H = diag(E_a + E_b + E_c) + sum_{i<j} g_ij P_i (x) P_j with per-child energies sorted U[0, 20],
    P_i = sym(N(0, 1)) / sqrt(d) and g_ij ~ U[0.05, 0.5], drawn from `rng` in that order (the
    energies of all three children, then the three port matrices, then each coupling as its term
    is formed).  Returns the oracle operator (dims d^3, N = d^3)."""
    Es = [np.sort(rng.uniform(0, 20, d)) for _ in range(3)]
    Ps = []
    for _ in range(3):
        A = rng.standard_normal((d, d))
        Ps.append((A + A.T) / 2 / np.sqrt(d))
    terms = [(1.0, [(a, kfref.DiagonalOp(Es[a]))]) for a in range(3)]
    for i, j in ((0, 1), (0, 2), (1, 2)):
        terms.append((rng.uniform(0.05, 0.5), [(i, kfref.DenseOp(Ps[i])), (j, kfref.DenseOp(Ps[j]))]))
    return kfref.KronFreeOperator([d, d, d], terms)


def real_three_oscillators(d):
    """Three truncated oscillators with real cos(0.5 (a + a')) pairwise couplings, restating the
    reference's test helper (test/helpers.jl:27-60): H = sum_i w_i n_i + 0.2 sum_{i<j} C_i C_j,
    w = (1.0, 1.1, 1.2), n = diag(0..d-1).  Returns (dims, terms with kfref ops)."""
    a = np.diag(np.sqrt(np.arange(1.0, d)), 1)
    X = a + a.T
    lam, V = np.linalg.eigh(X)
    cos_op = (V * np.cos(0.5 * lam)[None, :]) @ V.T
    nvec = np.arange(d, dtype=float)
    terms = [(w, [(i, kfref.DiagonalOp(nvec))]) for i, w in enumerate((1.0, 1.1, 1.2))]
    for i, j in ((0, 1), (1, 2), (0, 2)):
        terms.append((0.2, [(i, kfref.DenseOp(cos_op)), (j, kfref.DenseOp(cos_op))]))
    return [d, d, d], terms
