"""GPU parity of the operator application (kf_op_apply) against the oracle.

Cases follow the reference's test/test_apply.jl: every factor kind on every axis, blocks and
width changes, the fused diagonal and cancellation, extreme shifts and bands (out-of-range
offsets, zero shift, unsorted offsets), dense factors on first, middle and last axes, aliasing
and dimension errors.  FP64 results agree with the oracle to 1e-12 relative to ||H|| ||X||;
FP32 results to 2e-6 relative (FP32 storage, FP32 accumulation of at most ~20 terms).
"""
import numpy as np
import pytest

from oracle import circuits as ocirc
from oracle import kfref

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-6


def _to_oracle(op):
    from kfgpu import ops as P
    if isinstance(op, P.DenseOp):
        return kfref.DenseOp(op.M)
    if isinstance(op, P.DiagonalOp):
        return kfref.DiagonalOp(op.d)
    if isinstance(op, P.BandedOp):
        return kfref.BandedOp(op.n, op.offsets, op.weights)
    return kfref.ShiftOp(op.n, op.s, op.factor)


def _pair(dims, terms, constant=0.0, cap=1):
    from kfgpu import KronFreeOperator
    H = KronFreeOperator(dims, terms, constant=constant, block_capacity=cap)
    Ho = kfref.KronFreeOperator(dims, [(c, [(a, _to_oracle(op)) for a, op in fs]) for c, fs in terms],
                                constant=constant)
    return H, Ho


def _check(H, Ho, b=3, seed=0, f32=False):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((H.N, b))
    Y = H.apply(X.astype(np.float32) if f32 else X, f32=f32)
    R = Ho.matvec(X.astype(np.float32).astype(np.float64) if f32 else X)
    scale = max(1.0, np.max(np.abs(R)))
    err = np.max(np.abs(Y - R)) / scale
    assert err < (TOL32 if f32 else TOL64), err
    return err


def _random_op(kind, d, rng):
    from kfgpu import ops as P
    if kind == "dense":
        return P.DenseOp(rng.standard_normal((d, d)))
    if kind == "diag":
        return P.DiagonalOp(rng.standard_normal(d))
    if kind == "banded":
        return P.BandedOp(d, [-1, 0, 2], [rng.standard_normal(d) for _ in range(3)])
    return P.ShiftOp(d, 1, 0.7)


@pytest.mark.parametrize("kind", ["dense", "diag", "banded", "shift"])
@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("f32", [False, True])
def test_single_factor_every_axis(cuda, kind, axis, f32):
    rng = np.random.default_rng(hash((kind, axis)) % 2**32)
    dims = [3, 4, 5]
    H, Ho = _pair(dims, [(0.9, [(axis, _random_op(kind, dims[axis], rng))])], constant=0.25, cap=4)
    for b in (1, 4, 3):                                 # width changes (test/test_apply.jl:60-99)
        _check(H, Ho, b=b, seed=b, f32=f32)


@pytest.mark.parametrize("f32", [False, True])
def test_products_of_factors(cuda, f32):
    rng = np.random.default_rng(11)
    dims = [4, 5, 6]
    kinds = ["diag", "banded", "shift", "dense"]
    terms = []
    for k1 in kinds:
        for k2 in kinds:
            a1, a2 = 0, 2
            terms.append((rng.uniform(-1, 1), [(a1, _random_op(k1, dims[a1], rng)), (a2, _random_op(k2, dims[a2], rng))]))
    terms.append((0.3, [(0, _random_op("banded", 4, rng)), (1, _random_op("shift", 5, rng)), (2, _random_op("diag", 6, rng))]))
    H, Ho = _pair(dims, terms, constant=-1.5, cap=2)
    _check(H, Ho, b=5, f32=f32)


def test_fused_diagonal_and_cancellation(cuda):
    """test/test_apply.jl:120-140,184-229: all-diagonal terms fuse; opposite terms cancel exactly."""
    from kfgpu import ops as P
    d = np.arange(1.0, 6.0)
    terms = [(1.0, [(0, P.DiagonalOp(d))]), (-1.0, [(0, P.DiagonalOp(d))]),
             (2.0, [(0, P.DiagonalOp(d)), (1, P.DiagonalOp(np.ones(3)))])]
    H, Ho = _pair([5, 3], terms, constant=0.5)
    _check(H, Ho)
    assert np.allclose(H.diagonal(), Ho.full_diagonal(), atol=1e-14)


def test_extreme_shifts_and_bands(cuda):
    """Out-of-range offsets, zero shift, unsorted offsets (test/test_apply.jl:148-182)."""
    from kfgpu import ops as P
    rng = np.random.default_rng(5)
    d = 6
    terms = [
        (1.0, [(0, P.ShiftOp(d, 0, 2.0))]),
        (1.0, [(0, P.ShiftOp(d, 7, 1.0))]),             # shifts everything out
        (1.0, [(0, P.ShiftOp(d, -5, 3.0))]),
        (1.0, [(1, P.BandedOp(4, [3, -9, 0, -1], [rng.standard_normal(4) for _ in range(4)]))]),
        (0.5, [(0, P.BandedOp(d, [], [])), (1, P.DiagonalOp(rng.standard_normal(4)))]),
    ]
    H, Ho = _pair([d, 4], terms)
    _check(H, Ho, b=2)


def test_gershgorin_and_diagonal(cuda):
    from kfgpu import circuits
    th = ocirc.three_mode_theta(np.random.default_rng(3))
    dims, terms = circuits.three_mode_leaf(th, ncut=4, n2=16, n3=10)
    H, _ = _pair(dims, terms)
    Ho = ocirc.three_mode_operator(th, ncut=4, n2=16, n3=10)
    assert abs(H.gershgorin_bound() - Ho.gershgorin_bound()) < 1e-10 * Ho.gershgorin_bound()
    assert np.allclose(H.diagonal(), Ho.full_diagonal(), atol=1e-12)


@pytest.mark.parametrize("f32", [False, True])
def test_three_mode_leaf_reduced(cuda, f32):
    """The three-mode leaf Hamiltonian at a reduced size: GPU apply equals the spec-built oracle."""
    from kfgpu import circuits, KronFreeOperator
    th = ocirc.three_mode_theta(np.random.default_rng(1))
    dims, terms = circuits.three_mode_leaf(th, ncut=6, n2=40, n3=16)
    H = KronFreeOperator(dims, terms)
    Ho = ocirc.three_mode_operator(th, ncut=6, n2=40, n3=16)
    _check(H, Ho, b=16, f32=f32)


def test_three_mode_leaf_full_size(cuda):
    """N = 671,744 with a 16-column block: FP64 matches the oracle on every column; FP32 to 2e-6;
    symmetry <x, H y> = <H x, y> (a size-independent property)."""
    from kfgpu import circuits, KronFreeOperator
    th = ocirc.three_mode_theta(np.random.default_rng(20261205))
    dims, terms = circuits.three_mode_leaf(th)
    H = KronFreeOperator(dims, terms)
    Ho = ocirc.three_mode_operator(th)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((H.N, 16))
    Y = H.apply(X)
    R = Ho.matvec(X)
    assert np.max(np.abs(Y - R)) / np.max(np.abs(R)) < TOL64
    Y32 = H.apply(X.astype(np.float32), f32=True)
    R32 = Ho.matvec(X.astype(np.float32).astype(np.float64))
    assert np.max(np.abs(Y32 - R32)) / np.max(np.abs(R32)) < TOL32
    G = X.T @ Y
    assert np.max(np.abs(G - G.T)) < 1e-9 * np.max(np.abs(G))


def test_device_block_with_leading_dimension(cuda):
    """Column views of a larger block (ld > N) and the axpby epilogue on device buffers."""
    torch = cuda
    from kfgpu import circuits, KronFreeOperator
    th = ocirc.three_mode_theta(np.random.default_rng(2))
    dims, terms = circuits.three_mode_leaf(th, ncut=5, n2=24, n3=12)
    H = KronFreeOperator(dims, terms)
    Ho = ocirc.three_mode_operator(th, ncut=5, n2=24, n3=12)
    N, b, ld = H.N, 4, H.N + 37
    Xh = np.random.default_rng(4).standard_normal((ld, b))
    X = torch.tensor(Xh.T.copy(), device="cuda")          # row j of X is column j, stride ld
    Y = torch.zeros((b, ld), dtype=torch.float64, device="cuda")
    H.apply_device(X.data_ptr(), Y.data_ptr(), b, ldx=ld, ldy=ld)
    H.sync()
    R = Ho.matvec(Xh[:N, :])
    assert np.max(np.abs(Y.cpu().numpy()[:, :N].T - R)) < TOL64 * np.max(np.abs(R))
    # Chebyshev step: C = 2/e (H B - c B) - A
    A = torch.tensor(np.random.default_rng(5).standard_normal((b, N)), device="cuda")
    B = torch.tensor(np.random.default_rng(6).standard_normal((b, N)), device="cuda")
    Cc = torch.empty_like(A)
    c, e = 3.0, 7.0
    H.apply_axpby_device(B.data_ptr(), Cc.data_ptr(), A.data_ptr(), b, 2 / e, -2 * c / e, -1.0)
    H.sync()
    Bh, Ah = B.cpu().numpy().T, A.cpu().numpy().T
    ref = (2 / e) * (Ho.matvec(Bh) - c * Bh) - Ah
    assert np.max(np.abs(Cc.cpu().numpy().T - ref)) < TOL64 * np.max(np.abs(ref))


def test_errors(cuda):
    """Aliasing and dimension errors with the reference's messages (src/apply.jl:409-414, 226-231)."""
    torch = cuda
    from kfgpu import ArgumentError, DimensionMismatch, KronFreeOperator, ops as P
    H = KronFreeOperator([4, 3], [(1.0, [(0, P.ShiftOp(4, 1, 1.0))])])
    X = torch.zeros((2, 12), dtype=torch.float64, device="cuda")
    with pytest.raises(ArgumentError, match="alias"):
        H.apply_device(X.data_ptr(), X.data_ptr(), 2)
    with pytest.raises(DimensionMismatch):
        KronFreeOperator([4, 3], [(1.0, [(0, P.ShiftOp(5, 1, 1.0))])])
    with pytest.raises(ArgumentError, match="strictly increasing"):
        KronFreeOperator([4, 3], [(1.0, [(1, P.DiagonalOp(np.ones(3))), (0, P.DiagonalOp(np.ones(4)))])])
    with pytest.raises(ArgumentError, match="outside"):
        KronFreeOperator([4, 3], [(1.0, [(2, P.DiagonalOp(np.ones(3)))])])
    with pytest.raises(DimensionMismatch):
        H.apply(np.zeros((13, 1)))
    # an empty block is a no-op
    H.apply_device(X.data_ptr(), X.data_ptr() + 8 * 12, 0)


def _march_eligible(H, b, f32):
    import ctypes as C
    from kfgpu import _abi
    ok, g = C.c_int32(), (C.c_int32 * 16)()
    _abi.check(_abi.lib().kf_test_march_plan(H.handle, b, 1 if f32 else 0, 0, C.byref(ok), g))
    return ok.value == 1, list(g)


MARCH_SHAPES = ["three_mode", "wide", "outer", "mixed", "stencil3", "stencil7", "stencil9", "axes4"]


@pytest.mark.parametrize("f32", [False, True])
@pytest.mark.parametrize("shape", MARCH_SHAPES)
def test_plane_marching_apply(cuda, f32, shape):
    """The plane-marching kernel (variant 5: the slowest stencil axis from a register window, plane
    slices staged in shared memory by bulk copies, persistent CTAs) against the point-per-thread
    kernel and the oracle, forced past the autotuner: the three-mode structure, a plane wider than a
    tile, axes after the marching axis, entries with offsets on both the marching axis and an
    in-plane axis (and plane-dependent weights), 3-, 7- and 9-point stencils along the marching axis,
    and a 4-axis operator whose marching axis has nothing to march over (the point kernel runs)."""
    import ctypes as C
    torch = cuda
    from kfgpu import _abi, circuits, ops as P
    rng = np.random.default_rng(11)

    def banded(n, offs):
        return P.BandedOp(n, list(offs), [rng.standard_normal(n) for _ in offs])

    expect = True
    if shape == "three_mode":
        th = circuits.three_mode_theta(rng)
        dims, terms = circuits.three_mode_leaf(th, ncut=6, n2=48, n3=20)
    elif shape == "wide":
        dims = [41, 300, 5]
        terms = [(1.0, [(0, P.ShiftOp(41, 1, 1.0))]), (0.7, [(1, banded(300, (-2, -1, 0, 1, 2)))]),
                 (0.3, [(2, banded(5, (-1, 1)))]), (0.5, [(0, P.DiagonalOp(rng.standard_normal(41)))])]
    elif shape == "outer":
        dims = [41, 32, 20, 3]
        terms = [(1.0, [(1, banded(32, (-2, -1, 0, 1, 2)))]), (0.6, [(2, banded(20, (-2, -1, 0, 1, 2)))]),
                 (0.4, [(3, P.DiagonalOp(rng.standard_normal(3)))]),
                 (0.8, [(0, P.ShiftOp(41, -1, 1.0)), (3, P.DiagonalOp(rng.standard_normal(3)))]),
                 (0.2, [(2, banded(20, (-1, 1))), (3, P.DiagonalOp(rng.standard_normal(3)))])]
    elif shape == "mixed":
        dims = [24, 16, 30]
        terms = [(1.0, [(0, P.ShiftOp(24, 1, 1.0)), (2, banded(30, (-1, 0, 1)))]),
                 (0.5, [(0, P.DiagonalOp(rng.standard_normal(24))), (2, banded(30, (-2, 2)))]),
                 (0.7, [(1, banded(16, (-1, 1))), (2, P.DiagonalOp(rng.standard_normal(30)))]),
                 (0.3, [(2, banded(30, (-2, -1, 0, 1, 2)))]), (1.2, [(0, P.DiagonalOp(rng.standard_normal(24)))])]
    elif shape == "stencil3":
        dims = [33, 40, 24]
        terms = [(1.0, [(1, banded(40, (-1, 0, 1)))]), (0.9, [(2, banded(24, (-1, 0, 1)))]),
                 (0.5, [(0, P.ShiftOp(33, 1, 1.0))])]
    elif shape == "stencil7":
        dims = [20, 12, 40]
        terms = [(1.0, [(2, banded(40, tuple(range(-3, 4))))]), (0.5, [(0, banded(20, (-1, 1)))]),
                 (0.3, [(0, P.ShiftOp(20, 1, 1.0)), (2, banded(40, (-3, 3)))])]
    elif shape == "stencil9":
        dims = [64, 9, 30]
        terms = [(1.0, [(2, banded(30, tuple(range(-4, 5))))]), (0.5, [(1, banded(9, (-1, 1)))]),
                 (0.2, [(0, P.DiagonalOp(rng.standard_normal(64)))])]
    else:
        dims = [8, 20, 12, 3]
        terms = [(1.0, [(0, P.ShiftOp(8, -1, 2.0)), (1, banded(20, (-2, 0, 1)))]),
                 (0.4, [(3, P.DiagonalOp(rng.standard_normal(3)))]), (0.9, [(2, P.DiagonalOp(rng.standard_normal(12)))])]
        expect = False
    H, Ho = _pair(dims, terms)
    N, b = H.N, 5
    ok, geom = _march_eligible(H, b, f32)
    assert ok == expect, (shape, geom)
    dt = torch.float32 if f32 else torch.float64
    X = torch.as_tensor(rng.standard_normal((b, N)), dtype=dt, device="cuda")
    Ys = []
    flags = _abi.KF_DEVICE | (_abi.KF_F32 if f32 else _abi.KF_F64)
    for v in (0, 5, 7):
        Y = torch.full_like(X, float("nan"))
        _abi.check(_abi.lib().kf_test_apply_variant(H.handle, v, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), N,
                                                    b, flags, 1, None))
        Ys.append(Y.double().cpu().numpy())
    R = Ho.matvec(X.double().cpu().numpy().T).T
    scale = max(1.0, np.max(np.abs(R)))
    tol = TOL32 if f32 else TOL64
    for y in Ys[1:]:   # 5: 12 consumer warps, 7: 7 warps with twice the points per thread
        assert np.max(np.abs(y - R)) / scale < tol
        assert np.max(np.abs(y - Ys[0])) / scale < tol


@pytest.mark.parametrize("f32", [False, True])
def test_plane_marching_full_size(cuda, f32):
    """The marching kernel on the full three-mode leaf (41 x 256 x 64, 16 columns) against the
    oracle's C mul!, and with the Chebyshev epilogue Y = alpha H X + beta X + gamma Z through the
    tuned path."""
    import ctypes as C
    torch = cuda
    from kfgpu import _abi, circuits
    from oracle import capply
    rng = np.random.default_rng(5)
    th = circuits.three_mode_theta(rng)
    dims, terms = circuits.three_mode_leaf(th)
    H, Ho = _pair(dims, terms)
    N, b = H.N, 16
    ok, geom = _march_eligible(H, b, f32)
    assert ok and geom[:5] == [41 * 256, 64, 1, 2, 82], geom
    dt = torch.float32 if f32 else torch.float64
    X = torch.as_tensor(rng.standard_normal((b, N)), dtype=dt, device="cuda")
    flags = _abi.KF_DEVICE | (_abi.KF_F32 if f32 else _abi.KF_F64)
    Xh = np.asfortranarray(X.double().cpu().numpy().T)
    R = capply.CApply(Ho).matvec(Xh)
    scale = max(1.0, np.max(np.abs(R)))
    tol = TOL32 if f32 else TOL64
    for v in (5, 7):   # 12 consumer warps; 7 warps with twice the points per thread
        Y = torch.full_like(X, float("nan"))
        _abi.check(_abi.lib().kf_test_apply_variant(H.handle, v, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), N,
                                                    b, flags, 1, None))
        assert np.max(np.abs(Y.double().cpu().numpy().T - R)) / scale < tol, v
    # the epilogue, through the tuned kernel
    Zt = torch.as_tensor(rng.standard_normal((b, N)), dtype=dt, device="cuda")
    Y2 = torch.full_like(X, float("nan"))
    H.apply_axpby_device(X.data_ptr(), Y2.data_ptr(), Zt.data_ptr(), b, 0.5, -0.25, 2.0, f32=f32)
    H.sync()
    R2 = 0.5 * R - 0.25 * Xh + 2.0 * Zt.double().cpu().numpy().T
    assert np.max(np.abs(Y2.double().cpu().numpy().T - R2)) / max(1.0, np.max(np.abs(R2))) < tol


@pytest.mark.parametrize("f32", [False, True])
def test_every_point_variant_agrees(cuda, f32):
    """Every forced point-per-thread variant of the fused apply (0-4 and 6: the (columns per thread,
    unroll) shapes the tuner chooses from) gives the oracle's product on the three-mode structure,
    with more columns than one pass of the widest shape covers."""
    import ctypes as C
    torch = cuda
    from kfgpu import _abi, circuits
    rng = np.random.default_rng(23)
    th = circuits.three_mode_theta(rng)
    dims, terms = circuits.three_mode_leaf(th, ncut=6, n2=48, n3=20)
    H, Ho = _pair(dims, terms)
    N, b = H.N, 37
    dt = torch.float32 if f32 else torch.float64
    X = torch.as_tensor(rng.standard_normal((b, N)), dtype=dt, device="cuda")
    R = Ho.matvec(X.double().cpu().numpy().T).T
    scale = max(1.0, np.max(np.abs(R)))
    tol = TOL32 if f32 else TOL64
    flags = _abi.KF_DEVICE | (_abi.KF_F32 if f32 else _abi.KF_F64)
    for v in (0, 1, 2, 3, 4, 6):
        Y = torch.full_like(X, float("nan"))
        _abi.check(_abi.lib().kf_test_apply_variant(H.handle, v, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), N,
                                                    b, flags, 1, None))
        assert np.max(np.abs(Y.double().cpu().numpy() - R)) / scale < tol, v


@pytest.mark.parametrize("f32", [False, True])
@pytest.mark.parametrize("case", ["parent48", "distinct", "only02", "only12", "p01_p12", "banded", "d12"])
def test_dense_pair_terms(cuda, f32, case):
    """Dense pairwise couplings g A (x) B on a three-axis basis (the two-pass pair path: a mode
    product along the last axis, then per-slab register-blocked products) against the oracle's
    term-by-term mul!: shared and distinct factor matrices, every subset of pairs, an extra banded
    term (the fused pass first, the pairs accumulated), and the Chebyshev epilogue."""
    torch = cuda
    from kfgpu import ops as P
    rng = np.random.default_rng(101)
    d = 12 if case == "d12" else 48
    dims = [d, d, d]

    def sym(n):
        A = rng.standard_normal((n, n))
        return (A + A.T) / 2 / np.sqrt(n)

    Ps = [sym(d) for _ in range(3)]
    diag = [(1.0, [(a, P.DiagonalOp(np.sort(rng.uniform(0, 20, d))))]) for a in range(3)]
    pairs = {"01": (0.3, [(0, P.DenseOp(Ps[0])), (1, P.DenseOp(Ps[1]))]),
             "02": (0.2, [(0, P.DenseOp(Ps[0])), (2, P.DenseOp(Ps[2]))]),
             "12": (0.4, [(1, P.DenseOp(Ps[1])), (2, P.DenseOp(Ps[2]))])}
    if case == "distinct":
        pairs["02"] = (0.2, [(0, P.DenseOp(sym(d))), (2, P.DenseOp(Ps[2]))])
        pairs["12"] = (0.4, [(1, P.DenseOp(sym(d))), (2, P.DenseOp(sym(d)))])
    keys = {"only02": ["02"], "only12": ["12"], "p01_p12": ["01", "12"]}.get(case, ["01", "02", "12"])
    terms = diag + [pairs[k] for k in keys]
    if case == "banded":
        terms.append((0.7, [(1, P.BandedOp(d, [-1, 1], [rng.standard_normal(d), rng.standard_normal(d)]))]))
    H, Ho = _pair(dims, terms, cap=8)
    N, b = H.N, 6
    dt = torch.float32 if f32 else torch.float64
    X = torch.as_tensor(rng.standard_normal((b, N)), dtype=dt, device="cuda")
    Y = torch.full_like(X, float("nan"))
    H.apply_device(X.data_ptr(), Y.data_ptr(), b, f32=f32)
    H.sync()
    Xh = X.double().cpu().numpy().T
    R = Ho.matvec(Xh)
    tol = TOL32 if f32 else TOL64
    scale = max(1.0, np.max(np.abs(R)))
    assert np.max(np.abs(Y.double().cpu().numpy().T - R)) / scale < tol
    Zt = torch.as_tensor(rng.standard_normal((b, N)), dtype=dt, device="cuda")
    Y2 = torch.full_like(X, float("nan"))
    H.apply_axpby_device(X.data_ptr(), Y2.data_ptr(), Zt.data_ptr(), b, 0.5, -0.25, 2.0, f32=f32)
    H.sync()
    R2 = 0.5 * R - 0.25 * Xh + 2.0 * Zt.double().cpu().numpy().T
    assert np.max(np.abs(Y2.double().cpu().numpy().T - R2)) / max(1.0, np.max(np.abs(R2))) < tol
