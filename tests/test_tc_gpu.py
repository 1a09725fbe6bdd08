"""The tcgen05 tensor-core mode product (BF16 operands, FP32 accumulation in TMEM) against a
plain PyTorch FP32 reference of the same contraction, and the SIMT FP32 kernel against the same
reference: the axes of the three-mode leaf (41 x 256 x 64), of the dense parent (48^3), ragged
lengths that exercise the padding of M (to 128 / 256) and K (to a multiple of 16), several
column counts, alpha and accumulation into Y (beta = 1).

Tolerances: BF16 keeps 8 significant bits, so the BF16 tensor-core result is checked to 1e-2 of
the column norm (the separable preconditioner only steers search directions); the TF32 hi / lo
variant (the FP32 apply of dense factors, axes up to 96) to 2e-6, like the SIMT FP32 kernel (1e-5
here, 2e-6 in the apply tests).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ((41, 256, 64), 1, 16),
    ((41, 256, 64), 2, 16),
    ((41, 256, 64), 0, 3),
    ((48, 48, 48), 0, 8),
    ((48, 48, 48), 1, 8),
    ((48, 48, 48), 2, 8),
    ((37, 200, 3), 1, 5),
    ((130, 5), 0, 2),
    ((7, 129), 1, 1),
    ((16,), 0, 1),
    ((3, 256, 2), 1, 7),
    ((96, 5, 7), 0, 3),
    ((5, 64, 9), 1, 4),
]


def _reference(torch, X, A, dims, axis):
    """Y[l, i, r] = sum_j A[i, j] X[l, j, r] per column, in FP32 PyTorch."""
    b = X.shape[0]
    nd = len(dims)
    T = X.reshape((b,) + tuple(reversed(dims)))          # axis a is torch dim nd - a
    td = nd - axis
    At = torch.as_tensor(A, dtype=torch.float32, device=X.device)
    Y = torch.tensordot(T, At, dims=([td], [1]))           # contracted dim moves last
    Y = torch.movedim(Y, -1, td)
    return Y.reshape(b, -1).contiguous()


def _run(torch, path, X, A, dims, axis, alpha=1.0, beta=0.0, Y0=None):
    from kfgpu import _abi
    b, N = X.shape
    d = dims[axis]
    left = int(np.prod(dims[:axis])) if axis > 0 else 1
    Y = Y0.clone() if Y0 is not None else torch.zeros_like(X)
    Acol = np.ascontiguousarray(A.T, dtype=np.float64)    # column-major d x d
    st = _abi.lib().kf_test_mode_product(path, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                         Acol.ctypes.data_as(C.c_void_p), d, left, N, b, alpha, beta, None)
    _abi.check(st)
    return Y


@pytest.mark.parametrize("dims,axis,b", CASES)
def test_tensor_core_mode_product(cuda, dims, axis, b):
    torch = cuda
    rng = np.random.default_rng(hash((dims, axis, b)) % 2**32)
    d = dims[axis]
    N = int(np.prod(dims))
    A = rng.standard_normal((d, d)) / np.sqrt(d)
    X = torch.as_tensor(rng.standard_normal((b, N)), dtype=torch.float32, device="cuda")
    ref = _reference(torch, X, A, dims, axis)
    nref = torch.linalg.norm(ref, dim=1)
    Ys = _run(torch, 0, X, A, dims, axis)
    assert float(torch.max(torch.linalg.norm(Ys - ref, dim=1) / nref)) < 1e-5
    Yt = _run(torch, 1, X, A, dims, axis)
    err = torch.linalg.norm(Yt - ref, dim=1) / nref
    assert float(torch.max(err)) < 1e-2, err
    if d <= 96:
        # TF32 hi / lo operands, three MMAs per K step: FP32-level products
        Ys3 = _run(torch, 2, X, A, dims, axis)
        err3 = torch.linalg.norm(Ys3 - ref, dim=1) / nref
        assert float(torch.max(err3)) < 2e-6, err3


def test_tensor_core_alpha_beta(cuda):
    torch = cuda
    rng = np.random.default_rng(3)
    dims, axis, b = (41, 256, 64), 1, 4
    N = int(np.prod(dims))
    A = rng.standard_normal((256, 256)) / 16
    X = torch.as_tensor(rng.standard_normal((b, N)), dtype=torch.float32, device="cuda")
    Y0 = torch.as_tensor(rng.standard_normal((b, N)), dtype=torch.float32, device="cuda")
    ref = 0.5 * _reference(torch, X, A, dims, axis) + Y0
    Yt = _run(torch, 1, X, A, dims, axis, alpha=0.5, beta=1.0, Y0=Y0)
    err = torch.linalg.norm(Yt - ref, dim=1) / torch.linalg.norm(ref, dim=1)
    assert float(torch.max(err)) < 1e-2


def test_tensor_core_rejects_long_axis(cuda):
    torch = cuda
    from kfgpu._abi import ArgumentError
    X = torch.zeros((1, 300), dtype=torch.float32, device="cuda")
    with pytest.raises(ArgumentError):
        _run(torch, 1, X, np.eye(300), (300,), 0)
