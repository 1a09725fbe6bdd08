"""The FP32 Gram kernel (rows staged through shared memory, 8 x 8 tiles per warp, butterfly lane
reduction, fixed-order FP64 partial sums) against a plain PyTorch FP64 product of the same FP32
data: the shapes LOBPCG uses, ragged widths, the widest group layouts (1 x 8 and 8 x 1 tiles),
small N and a leading dimension larger than N (the scalar-copy path).  FP32 products summed in FP32
over at most ~70 rows per lane: 2e-6 of sqrt(sum|a|^2 sum|b|^2) per entry.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(16, 32, 671744), (32, 32, 671744), (1, 1, 1000), (2, 4, 3721), (7, 13, 5000), (8, 64, 20000),
          (64, 8, 20000), (48, 48, 110592), (128, 3, 4096), (5, 128, 300), (16, 16, 17)]


def _gram(A, B, N, path):
    """G = A' B of row-major torch blocks A (ka x N), B (kb x N) = column-major N x ka, N x kb."""
    from kfgpu import _abi
    ka, kb = A.shape[0], B.shape[0]
    G = np.zeros(ka * kb)
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_time_gram(path, C.c_void_p(A.data_ptr()), N, ka, C.c_void_p(B.data_ptr()), N,
                                            kb, N, 1, None, C.byref(ms), G.ctypes.data_as(C.c_void_p)))
    return G.reshape(kb, ka).T


@pytest.mark.parametrize("path", [0, 1])
@pytest.mark.parametrize("ka,kb,N", SHAPES)
def test_gram32_against_fp64(cuda, ka, kb, N, path):
    """path 1: the SIMT kernel; path 0: the solvers' dispatch (the tensor cores where they fit)."""
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(ka * 1000 + kb)
    A = torch.randn(ka, N, generator=g, device="cuda", dtype=torch.float32)
    B = torch.randn(kb, N, generator=g, device="cuda", dtype=torch.float32)
    G = _gram(A, B, N, path)
    ref = (A.double() @ B.double().T).cpu().numpy()
    scale = np.sqrt(np.outer((A.double() ** 2).sum(1).cpu().numpy(), (B.double() ** 2).sum(1).cpu().numpy()))
    assert np.max(np.abs(G - ref) / scale) < 2e-6


def test_gram32_leading_dimension(cuda):
    torch = cuda
    N, ld = 9999, 10003   # odd leading dimension: the 4-byte copy path
    g = torch.Generator(device="cuda").manual_seed(5)
    Abuf = torch.randn(6, ld, generator=g, device="cuda", dtype=torch.float32)
    Bbuf = torch.randn(9, ld, generator=g, device="cuda", dtype=torch.float32)
    from kfgpu import _abi
    G = np.zeros(6 * 9)
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_time_gram(1, C.c_void_p(Abuf.data_ptr()), ld, 6, C.c_void_p(Bbuf.data_ptr()), ld,
                                            9, N, 2, None, C.byref(ms), G.ctypes.data_as(C.c_void_p)))
    G = G.reshape(9, 6).T
    ref = (Abuf[:, :N].double() @ Bbuf[:, :N].double().T).cpu().numpy()
    assert np.max(np.abs(G - ref)) < 2e-6 * N
