"""The oracle against the reference's golden vectors and known-answer constructions.

Goldens: test/fixtures/scqubits_reference.json of KronFreeCircuits.jl (scqubits 4.3.1), with the
tolerances the reference's own tests use (test/test_materialize.jl:5-25,142-157,
test/test_zero_pi_reference.jl:21-55).
"""
import numpy as np
import pytest

from oracle import kfref, tree

PI = np.pi


def test_transmon_golden(goldens):
    g = goldens["goldens"]["transmon"]
    r = tree.materialize_leaf(goldens["specs"]["transmon"], g["params"], {"varphi_1": kfref.ChargeBasis(30)}, 5,
                              root=True)
    assert np.max(np.abs(r["energies"] - g["energies"])) < 1e-10


def test_fluxonium_golden(goldens):
    g = goldens["goldens"]["fluxonium"]
    r = tree.materialize_leaf(goldens["specs"]["fluxonium"], g["params"],
                              {"varphi_1": kfref.PhaseGrid(-10 * PI, 10 * PI, 1201, 8)}, 6, root=True)
    assert np.max(np.abs(r["energies"] - g["energies"])) < 1e-6


def test_zero_pi_small_golden(goldens):
    g = goldens["goldens"]["zero_pi_small"]
    r = tree.materialize_leaf(goldens["specs"]["zero_pi"], g["params"],
                              {"theta": kfref.ChargeBasis(6), "phi": kfref.PhaseGrid(-6 * PI, 6 * PI, 101, 6)}, 8,
                              root=True)
    assert np.max(np.abs(r["energies"] - g["energies"])) < 1e-9


def _two_transmon_tree(goldens):
    th = goldens["goldens"]["two_transmons"]["params"]
    return th, tree.materialize_branch(goldens["specs"]["two_transmons"], th,
                                       [{"varphi_1": kfref.ChargeBasis(30)}, {"varphi_2": kfref.ChargeBasis(30)}],
                                       [8, 8], 20)


def test_two_transmons_tree_golden(goldens):
    """The routed tree is a different truncation: lowest three to 1e-8, all twenty to 5e-4."""
    _, r = _two_transmon_tree(goldens)
    ref = np.array(goldens["goldens"]["two_transmons"]["energies"])
    assert np.max(np.abs(r["energies"][:3] - ref[:3])) < 1e-8
    assert np.max(np.abs(r["energies"] - ref)) < 5e-4


def test_two_transmons_bare_golden(goldens):
    th = goldens["goldens"]["two_transmons"]["params"]
    spec = goldens["specs"]["transmon"]

    def bare(EJ, EC, ng):
        return tree.materialize_leaf(spec, dict(E_J=EJ, E_C=EC, n_g=ng), {"varphi_1": kfref.ChargeBasis(30)}, 8,
                                     root=True, ports=[("varphi_1", "n")])
    b1, b2 = bare(th["E_J1"], th["E_C1"], th["n_g1"]), bare(th["E_J2"], th["E_C2"], th["n_g2"])
    n1, n2 = b1["ports"][("varphi_1", "n")], b2["ports"][("varphi_1", "n")]
    I = np.eye(8)
    H = np.kron(I, np.diag(b1["energies"])) + np.kron(np.diag(b2["energies"]), I) + \
        th["g"] * np.kron(n2 - th["n_g2"] * I, n1 - th["n_g1"] * I)
    ref = np.array(goldens["goldens"]["two_transmons"]["energies"])
    assert np.max(np.abs(np.linalg.eigvalsh(H)[:20] - ref)) < 1e-10


def test_branch_equals_explicit_product(goldens):
    """test/test_materialize.jl:117-125: the branch operator equals the explicit product construction."""
    th, r = _two_transmon_tree(goldens)
    q1, q2 = r["children"]
    P1 = tree._kept_port(q1, [("varphi_1", "n", 0.0)])
    P2 = tree._kept_port(q2, [("varphi_2", "n", 0.0)])
    I = np.eye(8)
    H = np.kron(I, np.diag(q1["energies"])) + np.kron(np.diag(q2["energies"]), I) + 0.3 * np.kron(P2, P1)
    c = kfref.constant_term(goldens["specs"]["two_transmons"], th)
    assert abs(c - 0.3) < 1e-14
    assert np.max(np.abs(np.linalg.eigvalsh(H)[:20] + c - r["energies"])) < 1e-10


def test_two_zero_pi_small_golden(goldens):
    thz = goldens["goldens"]["zero_pi_small"]["params"]
    leaf = tree.materialize_leaf(goldens["specs"]["zero_pi"], thz,
                                 {"theta": kfref.ChargeBasis(6), "phi": kfref.PhaseGrid(-6 * PI, 6 * PI, 101, 6)}, 10,
                                 root=True, ports=[("theta", "n")])
    D = np.diag(leaf["energies"])
    n = leaf["ports"][("theta", "n")] - thz["n_g"] * np.eye(10)
    I = np.eye(10)
    H = np.kron(I, D) + np.kron(D, I) + 0.05 * np.kron(n, n)
    ref = goldens["goldens"]["two_zero_pi_small"]["energies"]
    assert np.max(np.abs(np.linalg.eigvalsh(H)[:20] - ref)) < 1e-9


def test_two_zero_pi_small_ng0_tree_golden(goldens):
    th = goldens["goldens"]["two_zero_pi_small_ng0"]["params"]
    leaves = [{"theta1": kfref.ChargeBasis(6), "phi1": kfref.PhaseGrid(-6 * PI, 6 * PI, 101, 6)},
              {"theta2": kfref.ChargeBasis(6), "phi2": kfref.PhaseGrid(-6 * PI, 6 * PI, 101, 6)}]
    r = tree.materialize_branch(goldens["specs"]["two_zero_pi"], th, leaves, [10, 10], 20)
    assert np.max(np.abs(r["energies"] - goldens["goldens"]["two_zero_pi_small_ng0"]["energies"])) < 1e-9


def test_apply_matches_kron_reference():
    """test/test_apply.jl:5-58: every factor kind on every axis, blocks, against explicit krons."""
    rng = np.random.default_rng(3)
    dims = [3, 4, 5]
    ops = {
        "dense": lambda d: kfref.DenseOp(rng.standard_normal((d, d))),
        "diag": lambda d: kfref.DiagonalOp(rng.standard_normal(d)),
        "banded": lambda d: kfref.BandedOp(d, [-1, 0, 2], [rng.standard_normal(d) for _ in range(3)]),
        "shift": lambda d: kfref.ShiftOp(d, 1, 0.7),
    }
    for name, mk in ops.items():
        for a in range(3):
            terms = [(0.9, [(a, mk(dims[a]))])]
            H = kfref.KronFreeOperator(dims, terms, constant=0.25)
            X = rng.standard_normal((H.N, 3))
            ref = kfref.kron_reference(dims, terms, constant=0.25)
            assert np.allclose(H.matvec(X), ref @ X, atol=1e-12), (name, a)


def test_real_expansion_equals_complex():
    """cos(phi1 + phi2) + cos(phi1 - phi2) on charge x grid: real by structure; the summed real
    expansions (src/character.jl:297-315) equal the complex operator."""
    b = kfref.PhaseGrid(-PI, PI, 9, 2)
    c = kfref.ChargeBasis(2)
    terms = []
    for s1, s2 in ((1, 1), (-1, -1), (1, -1), (-1, 1)):
        terms.append((-0.5, [(0, kfref.localop(c, "expiphi", s1)), (1, kfref.localop(b, "expiphi", s2))]))
    dims = [5, 9]
    full = kfref.kron_reference(dims, terms)
    real_terms = [rt for c0, fs in terms for rt in kfref.real_expansion(c0, fs)]
    rr = kfref.kron_reference(dims, real_terms)
    assert np.allclose(full.imag, 0, atol=1e-14)
    assert np.allclose(rr, full.real, atol=1e-14)
