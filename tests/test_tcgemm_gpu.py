"""The tcgen05 block update (TF32 hi / lo operands, hi*hi + hi*lo + lo*hi in two MMAs per K step,
warp-specialised pipeline) and the SIMT update against a plain PyTorch FP64 product of the same FP32
data: LOBPCG's
shapes (the fused orthogonalisation update [Z X] -> Z at 32 + 16 -> 32 columns, the Rayleigh-Ritz
updates), ragged row counts (not a multiple of the 128-row tile), wide outputs, leading dimensions
larger than N, alpha and accumulation into Y.  FP32 results: 5e-6 of sum_i |X_ri| |C_ij| per entry.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(671744, 32, 16, 32), (671744, 36, 18, 36), (671744, 16, 0, 16), (3721, 7, 0, 5), (1000, 48, 16, 80),
          (129, 3, 2, 1), (20000, 64, 0, 17), (300, 1, 0, 80)]


def _update(torch, path, X0, X1, Cm, Y0, alpha, beta, ld, N):
    from kfgpu import _abi
    kx0, kx1, ky = X0.shape[0], (X1.shape[0] if X1 is not None else 0), Cm.shape[1]
    Y = Y0.clone()
    Ch = np.asfortranarray(Cm)
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_update(path, C.c_void_p(Y.data_ptr()), ld, ky, C.c_void_p(X0.data_ptr()), ld, kx0,
                                         C.c_void_p(X1.data_ptr()) if X1 is not None else None, ld, kx1,
                                         Ch.ctypes.data_as(C.c_void_p), Cm.shape[0], alpha, beta, N, 1, None,
                                         C.byref(ms)))
    return Y


@pytest.mark.parametrize("N,kx0,kx1,ky", SHAPES)
@pytest.mark.parametrize("path", [0, 1])
def test_block_update(cuda, path, N, kx0, kx1, ky):
    torch = cuda
    rng = np.random.default_rng(N + 7 * kx0 + ky)
    ld = N + (5 if N % 2 else 0)
    # blocks as (columns, ld) torch arrays: column-major N x k with leading dimension ld
    X0 = torch.as_tensor(rng.standard_normal((kx0, ld)), dtype=torch.float32, device="cuda")
    X1 = torch.as_tensor(rng.standard_normal((kx1, ld)), dtype=torch.float32, device="cuda") if kx1 else None
    Cm = rng.standard_normal((kx0 + kx1, ky))
    Y0 = torch.as_tensor(rng.standard_normal((ky, ld)), dtype=torch.float32, device="cuda")
    for alpha, beta in ((1.0, 0.0), (-0.5, 1.0)):
        Y = _update(torch, path, X0, X1, Cm, Y0, alpha, beta, ld, N)
        Xa = X0[:, :N] if X1 is None else torch.cat([X0[:, :N], X1[:, :N]])
        Cf = Cm.astype(np.float32).astype(np.float64)          # the kernels round C to FP32 first
        Ct = torch.as_tensor(Cf, dtype=torch.float64, device="cuda")
        ref = alpha * (Ct.T @ Xa.double()) + beta * Y0[:, :N].double()
        bound = abs(alpha) * (torch.as_tensor(np.abs(Cf), device="cuda").T @ Xa.double().abs()) + \
            abs(beta) * Y0[:, :N].double().abs() + 1e-30
        err = ((Y[:, :N].double() - ref).abs() / bound).max().item()
        assert err < 5e-6, (path, alpha, beta, err)
        # the padding rows of each column (ld > N) are untouched
        if ld > N:
            assert torch.equal(Y[:, N:], Y0[:, N:])


def test_tensor_core_update_rejects_wide_outputs(cuda):
    """Two accumulator slots of 3 Np columns fit TMEM up to 80 outputs; wider updates are refused
    (the solvers keep the SIMT kernels there)."""
    torch = cuda
    from kfgpu._abi import ArgumentError
    X0 = torch.zeros((8, 1024), dtype=torch.float32, device="cuda")
    Y0 = torch.zeros((96, 1024), dtype=torch.float32, device="cuda")
    with pytest.raises(ArgumentError):
        _update(torch, 1, X0, None, np.zeros((8, 96)), Y0, 1.0, 0.0, 1024, 1024)


RING_SHAPES = [(671744, 18, 36, 36), (671744, 18, 36, 18), (100003, 7, 0, 5), (129, 3, 2, 1), (20000, 64, 0, 17),
               (300, 1, 0, 80), (5000, 48, 16, 80)]


def _ring_smem(kx, ky, nstg):
    """Shared memory of the tensor-core update with an nstg-tile staging ring (bytes)."""
    Kp, Np = (kx + 7) // 8 * 8, (ky + 15) // 16 * 16
    return 2 * Np * Kp * 4 + 4 * 128 * Kp * 4 + 128 + nstg * Kp * 132 * 4


@pytest.mark.parametrize("N,kx0,kx1,ky", RING_SHAPES)
@pytest.mark.parametrize("path", [2, 3, 4])
def test_block_update_producer_modes(cuda, path, N, kx0, kx1, ky):
    """The tensor-core update with its producer mode forced: register gather (path 2), staging rings
    of two and three tiles filled by 16-byte cp.async copies (paths 3, 4; the rows past N of the last
    tile zero-filled).  A ring that does not fit shared memory is refused."""
    torch = cuda
    from kfgpu._abi import ArgumentError
    rng = np.random.default_rng(N + 3 * kx0 + ky)
    ld = (N + 3) // 4 * 4 + (4 if N % 3 == 0 else 0)
    X0 = torch.as_tensor(rng.standard_normal((kx0, ld)), dtype=torch.float32, device="cuda")
    X1 = torch.as_tensor(rng.standard_normal((kx1, ld)), dtype=torch.float32, device="cuda") if kx1 else None
    Cm = rng.standard_normal((kx0 + kx1, ky))
    Y0 = torch.as_tensor(rng.standard_normal((ky, ld)), dtype=torch.float32, device="cuda")
    smem = _ring_smem(kx0 + kx1, ky, path - 1) if path >= 3 else 0
    if smem > 232448:
        with pytest.raises(ArgumentError):
            _update(torch, path, X0, X1, Cm, Y0, 1.0, 0.0, ld, N)
        return
    for alpha, beta in ((1.0, 0.0), (0.75, -1.0)):
        Y = _update(torch, path, X0, X1, Cm, Y0, alpha, beta, ld, N)
        Xa = X0[:, :N] if X1 is None else torch.cat([X0[:, :N], X1[:, :N]])
        Cf = Cm.astype(np.float32).astype(np.float64)
        Ct = torch.as_tensor(Cf, dtype=torch.float64, device="cuda")
        ref = alpha * (Ct.T @ Xa.double()) + beta * Y0[:, :N].double()
        bound = abs(alpha) * (torch.as_tensor(np.abs(Cf), device="cuda").T @ Xa.double().abs()) + \
            abs(beta) * Y0[:, :N].double().abs() + 1e-30
        err = ((Y[:, :N].double() - ref).abs() / bound).max().item()
        assert err < 5e-6, (path, alpha, beta, err)
        if ld > N:
            assert torch.equal(Y[:, N:], Y0[:, N:])
