"""Term lists of the measured circuits, built from `kfgpu.ops` ports (real components).

These are the AxisTerm lists the reference's `_node_operator` hands to `KronFreeOperator` for
each node (src/materialize.jl:583-647); here they are written out per circuit.

  three_mode_leaf      41 x 256 x 64 charge x grid x grid leaf (N = 671,744)
  fluxonium_leaf       a 1-D phase-grid leaf of n points on [-5 pi, 5 pi]
  transmon_leaf        a charge-basis transmon leaf (ChargeBasis(30))
  two_transmon_flat    the two-transmon circuit on the flat 61 x 61 product space
  dense_parent         a three-child parent with dense port couplings (48^3 = 110,592)
"""
from __future__ import annotations

import numpy as np

from .ops import ChargeBasis, DenseOp, DiagonalOp, PhaseGrid, ShiftOp, localop

PI = np.pi


def three_mode_bases(ncut=20, n2=256, n3=64):
    return [ChargeBasis(ncut), PhaseGrid(-4 * PI, 4 * PI, n2, 4), PhaseGrid(-3 * PI, 3 * PI, n3, 4)]


def three_mode_theta(rng):
    """theta ~ U: E_J [5,15], E_C1 [0.02,0.1], E_C2, E_C3 [0.5,2], E_L [0.02,0.2], E_J' [0.5,2]."""
    return {"E_J": rng.uniform(5, 15), "E_C1": rng.uniform(0.02, 0.1), "E_C2": rng.uniform(0.5, 2),
            "E_C3": rng.uniform(0.5, 2), "E_L": rng.uniform(0.02, 0.2), "E_Jp": rng.uniform(0.5, 2)}


def three_mode_leaf(theta, ncut=20, n2=256, n3=64):
    """H = 4E_C1 n1^2 - E_C2 d2^2 - E_C3 d3^2 + E_L/2 (phi2^2 + phi3^2) - 2E_J cos phi1 cos phi2 - E_J' cos(phi2 - phi3).

    Returns (dims, terms).  2 cos phi1 = S+ + S- on the charge axis; cos(phi2 - phi3) =
    cos2 cos3 + sin2 sin3 (both diagonal, so fused into the diagonal by the library).
    """
    b1, b2, b3 = three_mode_bases(ncut, n2, n3)
    t = theta
    terms = [
        (4 * t["E_C1"], [(0, localop(b1, "n2"))]),
        (t["E_C2"], [(1, localop(b2, "n2"))]),
        (t["E_C3"], [(2, localop(b3, "n2"))]),
        (t["E_L"] / 2, [(1, localop(b2, "phi2"))]),
        (t["E_L"] / 2, [(2, localop(b3, "phi2"))]),
        (-t["E_J"], [(0, localop(b1, "expiphi", 1)), (1, localop(b2, "expiphi", 1, "re"))]),
        (-t["E_J"], [(0, localop(b1, "expiphi", -1)), (1, localop(b2, "expiphi", 1, "re"))]),
        (-t["E_Jp"], [(1, localop(b2, "expiphi", 1, "re")), (2, localop(b3, "expiphi", 1, "re"))]),
        (-t["E_Jp"], [(1, localop(b2, "expiphi", 1, "im")), (2, localop(b3, "expiphi", 1, "im"))]),
    ]
    return [b.dim for b in (b1, b2, b3)], terms


def fluxonium_theta(rng):
    """E_J [3,10], E_C [0.5,1.5], E_L [0.2,1.2], phi_ext [0, 2 pi]."""
    return {"E_J": rng.uniform(3, 10), "E_C": rng.uniform(0.5, 1.5), "E_L": rng.uniform(0.2, 1.2),
            "phi_ext": rng.uniform(0, 2 * PI)}


def fluxonium_leaf(theta, npts):
    """H = -E_C d^2 (5-point) + E_L/2 phi^2 - E_J cos(phi - phi_ext) on npts points of [-5 pi, 5 pi]."""
    b = PhaseGrid(-5 * PI, 5 * PI, npts, 4)
    t = theta
    ce, se = np.cos(t["phi_ext"]), np.sin(t["phi_ext"])
    terms = [
        (t["E_C"], [(0, localop(b, "n2"))]),
        (t["E_L"] / 2, [(0, localop(b, "phi2"))]),
        (-t["E_J"] * ce, [(0, localop(b, "expiphi", 1, "re"))]),
        (-t["E_J"] * se, [(0, localop(b, "expiphi", 1, "im"))]),
    ]
    return [npts], terms


def transmon_terms(E_J, E_C, n_g, axis=0, ncut=30, lin_extra=0.0):
    """4E_C (n - n_g)^2 - E_J cos phi without its constant: 4E_C n^2 - 8 E_C n_g n - E_J/2 (S+ + S-)."""
    b = ChargeBasis(ncut)
    return [
        (4 * E_C, [(axis, localop(b, "n2"))]),
        (-8 * E_C * n_g + lin_extra, [(axis, localop(b, "n"))]),
        (-E_J / 2, [(axis, localop(b, "expiphi", 1))]),
        (-E_J / 2, [(axis, localop(b, "expiphi", -1))]),
    ]


def two_transmon_flat(theta, ncut=30):
    """The two-transmon circuit with E_C off-diagonal g/8 on the flat product of two charge bases.

    g (n1 - n_g1)(n2 - n_g2) = g n1 n2 - g n_g2 n1 - g n_g1 n2 + g n_g1 n_g2 (the constant is
    returned separately, with 4 n_g' E_C n_g).
    """
    t = theta
    b = ChargeBasis(ncut)
    terms = transmon_terms(t["E_J1"], t["E_C1"], t["n_g1"], 0, ncut, lin_extra=-t["g"] * t["n_g2"]) + \
        transmon_terms(t["E_J2"], t["E_C2"], t["n_g2"], 1, ncut, lin_extra=-t["g"] * t["n_g1"])
    terms.append((t["g"], [(0, localop(b, "n")), (1, localop(b, "n"))]))
    EC = np.array([[t["E_C1"], t["g"] / 8], [t["g"] / 8, t["E_C2"]]])
    ng = np.array([t["n_g1"], t["n_g2"]])
    return [b.dim, b.dim], terms, float(4 * ng @ EC @ ng)


def dense_parent(rng, d=48):
    """Three children keeping d states: diag(E_a + E_b + E_c) + sum_{i<j} g_ij P_i (x) P_j.

    E sorted U[0, 20]; P_i = sym(N(0,1)) / sqrt(d); g ~ U[0.05, 0.5].
    """
    Es = [np.sort(rng.uniform(0, 20, d)) for _ in range(3)]
    Ps = []
    for _ in range(3):
        A = rng.standard_normal((d, d))
        Ps.append((A + A.T) / 2 / np.sqrt(d))
    terms = [(1.0, [(a, DiagonalOp(Es[a]))]) for a in range(3)]
    for i, j in ((0, 1), (0, 2), (1, 2)):
        terms.append((rng.uniform(0.05, 0.5), [(i, DenseOp(Ps[i])), (j, DenseOp(Ps[j]))]))
    return [d, d, d], terms
