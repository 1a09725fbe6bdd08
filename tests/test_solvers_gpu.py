"""GPU eigensolvers (kf_solve) against the FP64 oracle.

The reference pins its solvers at the boundary: eigenvalues equal Dense's, every true residual is
below tol, the vectors are orthonormal (test/helpers.jl:128-135, test/test_solvers.jl:4-14,688,
test/cuda/test_device.jl:62-131).  Here: eigenvalues within 1e-9 relative of the oracle's Dense
(LAPACK) values, residuals ||H v - E v|| recomputed by the oracle's own operator below tol,
||V'V - I|| < 1e-10, for FP64 and mixed precision.
"""
import numpy as np
import pytest

from oracle import circuits as ocirc
from oracle import kfref, solvers as osol

pytestmark = pytest.mark.gpu


def _check_pairs(Ho, E, V, Eref, tol, rel=1e-9):
    assert np.max(np.abs(E - Eref) / np.maximum(1.0, np.abs(Eref))) < rel, np.abs(E - Eref)
    R = Ho.matvec(V) - V * E[None, :]
    res = np.sqrt(np.sum(R ** 2, axis=0))
    assert np.max(res) <= tol, res
    assert np.linalg.norm(V.T @ V - np.eye(V.shape[1])) < 1e-10


@pytest.fixture(scope="module")
def small_leaf():
    from kfgpu import circuits, KronFreeOperator
    th = ocirc.three_mode_theta(np.random.default_rng(12))
    kw = dict(ncut=5, n2=24, n3=12)
    dims, terms = circuits.three_mode_leaf(th, **kw)
    Ho = ocirc.three_mode_operator(th, **kw)
    Eref, _ = osol.dense_solve(Ho, 16)
    return KronFreeOperator(dims, terms), Ho, Eref


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_lobpcg_matches_dense(cuda, small_leaf, precision):
    from kfgpu import LOBPCG, solve
    H, Ho, Eref = small_leaf
    tol = 1e-8 * H.gershgorin_bound()
    E, V, st = solve(LOBPCG(tol=tol, precision=precision), H, 12)
    _check_pairs(Ho, E, V, Eref[:12], tol)
    assert st["converged"] == 12 and st["n_matvec"] > 0


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_chebyshev_matches_dense(cuda, small_leaf, precision):
    from kfgpu import ChebyshevFilter, solve
    H, Ho, Eref = small_leaf
    tol = 1e-8 * H.gershgorin_bound()
    E, V, st = solve(ChebyshevFilter(tol=tol, degree=20, extra=8, precision=precision), H, 12)
    _check_pairs(Ho, E, V, Eref[:12], tol * 1.0001)


def test_chebyshev_weak_filter_raises_like_the_oracle(cuda, small_leaf):
    """degree 20 with extra 4 is a weak filter on this leaf: the oracle runs out of maxiter = 50
    (14 of 15 locked), and so must the GPU solver, with the reference's maxiter error."""
    from kfgpu import ChebyshevFilter, ConvergenceError, solve
    H, Ho, Eref = small_leaf
    with pytest.raises(ConvergenceError, match="within maxiter = 50"):
        solve(ChebyshevFilter(tol=1e-8 * H.gershgorin_bound(), degree=20, extra=4), H, 12)


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_lobpcg_separable_preconditioner(cuda, small_leaf, precision):
    """The separable preconditioner (per-axis eigenbases of the single-axis terms) gives the Dense pairs."""
    from kfgpu import LOBPCG, solve
    H, Ho, Eref = small_leaf
    tol = 1e-8 * H.gershgorin_bound()
    E, V, st = solve(LOBPCG(tol=tol, precision=precision, preconditioner="separable"), H, 12)
    _check_pairs(Ho, E, V, Eref[:12], tol)


def test_separable_preconditioner_on_a_stiff_grid(cuda):
    """On a fine grid (||H|| dominated by the 1/Delta^2 stencils) the separable preconditioner
    converges in a fraction of the per-Ritz Jacobi iterations, to the same eigenvalues (1e-9 rel)."""
    from kfgpu import KronFreeOperator, LOBPCG, circuits, solve
    th = ocirc.three_mode_theta(np.random.default_rng(20261205))
    dims, terms = circuits.three_mode_leaf(th, ncut=8, n2=128, n3=32)
    H = KronFreeOperator(dims, terms)
    tol = 1e-8 * H.gershgorin_bound()
    Es, Vs, ss = solve(LOBPCG(tol=tol, preconditioner="separable"), H, 8)
    Er, Vr, sr = solve(LOBPCG(tol=tol), H, 8)
    assert np.max(np.abs(Es - Er) / np.abs(Er)) < 1e-9
    assert ss["iterations"] < 0.5 * sr["iterations"]
    Ho = ocirc.three_mode_operator(th, ncut=8, n2=128, n3=32)
    R = Ho.matvec(Vs) - Vs * Es[None, :]
    assert np.max(np.sqrt(np.sum(R ** 2, axis=0))) <= tol


def test_lobpcg_warm_start_and_random_seed(cuda, small_leaf):
    from kfgpu import LOBPCG, solve
    H, Ho, Eref = small_leaf
    tol = 1e-8 * H.gershgorin_bound()
    E, V, st = solve(LOBPCG(tol=tol), H, 8)
    E2, V2, st2 = solve(LOBPCG(tol=tol), H, 8, X0=V)
    _check_pairs(Ho, E2, V2, Eref[:8], tol)
    # work in H columns, as the reference measures it (test/test_solvers.jl:798): the guards
    # converge alike on warm and cold starts, but the seeded columns lock at once
    assert st2["warm"] == 1 and st2["n_matvec"] < st["n_matvec"]
    E3, V3, _ = solve(LOBPCG(tol=tol, seed="random", preconditioner="jacobi"), H, 8)
    _check_pairs(Ho, E3, V3, Eref[:8], tol)


def test_lobpcg_argument_and_convergence_errors(cuda, small_leaf):
    from kfgpu import ArgumentError, ConvergenceError, KronFreeOperator, LOBPCG, solve, ops as P
    H, Ho, _ = small_leaf
    small = KronFreeOperator([10], [(1.0, [(0, P.DiagonalOp(np.arange(10.0)))])])
    with pytest.raises(ArgumentError, match="3m \\+ 5"):
        solve(LOBPCG(), small, 3)
    X0 = np.random.default_rng(0).standard_normal((H.N, 4))
    X0[:, 2] = 0
    with pytest.raises(ArgumentError, match="column 3 of X0 is zero"):
        solve(LOBPCG(), H, 4, X0=X0)
    X0[:, 2] = np.nan
    with pytest.raises(ArgumentError, match="non-finite"):
        solve(LOBPCG(), H, 4, X0=X0)
    with pytest.raises(ConvergenceError, match="did not converge"):
        solve(LOBPCG(tol=1e-12, maxiter=1), H, 4)


def test_pathological_identity_and_zero(cuda):
    """S1/S2 of the reference's catalogue (test/test_solvers.jl:903-1104): H = cI breaks a
    product-seed LOBPCG (an exactly zero residual block) and must raise, never return garbage;
    Chebyshev on a one-axis diagonal operator returns exact pairs."""
    from kfgpu import ChebyshevFilter, ConvergenceError, KronFreeOperator, LOBPCG, solve, ops as P
    n = 64
    H = KronFreeOperator([n], [(1.0, [(0, P.DiagonalOp(np.linspace(0, 5, n)))])])
    E, V, _ = solve(ChebyshevFilter(degree=10, extra=4), H, 5)
    assert np.allclose(E, np.linspace(0, 5, n)[:5], atol=1e-12)
    Hc = KronFreeOperator([n], [], constant=2.0)
    try:
        E, V, _ = solve(LOBPCG(), Hc, 4)
        assert np.allclose(E, 2.0)
    except ConvergenceError:
        pass


def _to_oracle(op):
    from kfgpu import ops as P
    if isinstance(op, P.DenseOp):
        return kfref.DenseOp(op.M)
    return kfref.DiagonalOp(op.d)


def test_dense_parent_lobpcg(cuda):
    """A parent with dense port couplings (three children, d = 12): LOBPCG vs Dense, both precisions."""
    from kfgpu import circuits, KronFreeOperator, LOBPCG, solve
    dims, terms = circuits.dense_parent(np.random.default_rng(4), d=12)
    H = KronFreeOperator(dims, terms, block_capacity=12)
    Ho = kfref.KronFreeOperator(dims, [(c, [(a, _to_oracle(op)) for a, op in fs]) for c, fs in terms])
    Eref, _ = osol.dense_solve(Ho, 10)
    for prec in ("f64", "mixed"):
        tol = 1e-8 * H.gershgorin_bound()
        E, V, _ = solve(LOBPCG(tol=tol, guard=2, precision=prec), H, 10)
        _check_pairs(Ho, E, V, Eref[:10], tol)


def test_two_transmons_via_gpu_matrix(cuda, goldens):
    """The two-transmon tree with every node's Matrix(H) formed by GPU applies on identity blocks
    (the reference's Dense path, src/apply.jl:506-531): leaves keep 8, top keeps 20; energies
    against the scqubits golden (lowest 3 to 1e-8, all to 5e-4) and the oracle tree (1e-10)."""
    from kfgpu import circuits, KronFreeOperator, ops as P
    from oracle import tree
    th = goldens["goldens"]["two_transmons"]["params"]

    def gpu_matrix(dims, terms, const=0.0):
        H = KronFreeOperator(dims, terms, constant=const, block_capacity=256)
        return H.apply(np.eye(H.N))

    leaves = []
    for i, (EJ, EC, ng, lin) in enumerate([(th["E_J1"], th["E_C1"], th["n_g1"], -th["g"] * th["n_g2"]),
                                           (th["E_J2"], th["E_C2"], th["n_g2"], -th["g"] * th["n_g1"])]):
        M = gpu_matrix([61], circuits.transmon_terms(EJ, EC, ng, 0, 30, lin_extra=lin))
        w, V = np.linalg.eigh((M + M.T) / 2)
        n = np.arange(-30.0, 31.0)
        leaves.append((w[:8], V[:, :8].T @ (n[:, None] * V[:, :8])))
    EC = np.array([[th["E_C1"], th["g"] / 8], [th["g"] / 8, th["E_C2"]]])
    ng = np.array([th["n_g1"], th["n_g2"]])
    const = float(4 * ng @ EC @ ng)
    terms = [(1.0, [(0, P.DiagonalOp(leaves[0][0]))]), (1.0, [(1, P.DiagonalOp(leaves[1][0]))]),
             (th["g"], [(0, P.DenseOp(leaves[0][1])), (1, P.DenseOp(leaves[1][1]))])]
    M = gpu_matrix([8, 8], terms, const)
    E = np.linalg.eigvalsh((M + M.T) / 2)[:20]
    ref = np.array(goldens["goldens"]["two_transmons"]["energies"])
    assert np.max(np.abs(E[:3] - ref[:3])) < 1e-8
    assert np.max(np.abs(E - ref)) < 5e-4
    o = tree.materialize_branch(goldens["specs"]["two_transmons"], th,
                                [{"varphi_1": kfref.ChargeBasis(30)}, {"varphi_2": kfref.ChargeBasis(30)}], [8, 8], 20)
    assert np.max(np.abs(E - o["energies"])) < 1e-10


def test_three_mode_leaf_full_size_mixed_vs_f64(cuda):
    """N = 671,744, m = 12, block 16: mixed-precision LOBPCG against plain FP64 LOBPCG (eigenvalues
    within 1e-9 relative) with every residual <= 1e-8 ||H|| recomputed by the oracle's operator."""
    from kfgpu import circuits, KronFreeOperator, LOBPCG, solve
    th = ocirc.three_mode_theta(np.random.default_rng(20261205))
    dims, terms = circuits.three_mode_leaf(th)
    H = KronFreeOperator(dims, terms)
    tol = 1e-8 * H.gershgorin_bound()
    E64, V64, s64 = solve(LOBPCG(tol=tol), H, 12)
    Em, Vm, sm = solve(LOBPCG(tol=tol, precision="mixed"), H, 12)
    assert np.max(np.abs(Em - E64) / np.abs(E64)) < 1e-9
    Ho = ocirc.three_mode_operator(th)
    for E, V in ((E64, V64), (Em, Vm)):
        R = Ho.matvec(V) - V * E[None, :]
        assert np.max(np.sqrt(np.sum(R ** 2, axis=0))) <= tol


def test_device_product_seed_matches_host(cuda):
    """kf_op_product_seed (product_seed, src/apply.jl:655-685, built on the device) spans the same
    states as the host mirror: orthonormal columns, the same product states up to sign (the
    per-axis eigenvectors' signs are free)."""
    from kfgpu import KronFreeOperator, ArgumentError, circuits, ops as P
    th = circuits.three_mode_theta(np.random.default_rng(8))
    dims, terms = circuits.three_mode_leaf(th, ncut=6, n2=48, n3=20)
    H = KronFreeOperator(dims, terms)
    for k in (1, 16, 40):
        Xd = H.product_seed_device(k)
        Xh = H.product_seed(k)
        assert np.allclose(Xd.T @ Xd, np.eye(k), atol=1e-12)
        assert np.allclose(np.abs(np.sum(Xd * Xh, axis=0)), 1.0, atol=1e-9)
    with pytest.raises(ArgumentError, match="product_seed: k must lie in"):
        H.product_seed_device(H.N + 1)
    # every axis diagonal: unit vectors at the smallest entries of the full diagonal
    D = KronFreeOperator([7, 5], [(1.0, [(0, P.DiagonalOp(np.arange(7.0)[::-1]))]),
                                  (0.5, [(1, P.DiagonalOp(np.arange(5.0)))])])
    assert np.array_equal(D.product_seed_device(4), D.product_seed(4))
