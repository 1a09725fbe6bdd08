"""The FP64 block update Y = X C of the refinement's large-rotation step, as the FP64 kernel and in
double-float arithmetic on the FP32 pipes, against a PyTorch FP64 product: the widths of the
three-mode leaf's block (16 + guards + buffers), the largest supported (32), ragged ones and a
single column.  Double-float keeps about 46 bits: 1e-13 of sqrt(sum_i x_i^2 c_ij^2)-scale per entry
(here of the row norm times the column norm), well below the 1e-8 residual target of the solve."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(torch, path, X, Cm):
    from kfgpu import _abi
    kx, N = X.shape
    ky = Cm.shape[1]
    Y = torch.zeros((ky, N), dtype=torch.float64, device="cuda")
    Cf = np.asfortranarray(Cm)
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_update_f64(path, C.c_void_p(Y.data_ptr()), C.c_void_p(X.data_ptr()), kx, ky,
                                             Cf.ctypes.data_as(C.c_void_p), N, 2, None, C.byref(ms)))
    return Y


@pytest.mark.parametrize("kx,ky,N", [(18, 18, 671744), (32, 32, 100000), (16, 16, 4096), (7, 5, 3001), (1, 1, 17),
                                     (20, 3, 50000)])
def test_update_f64_paths(cuda, kx, ky, N):
    torch = cuda
    rng = np.random.default_rng(kx * 100 + ky)
    g = torch.Generator(device="cuda").manual_seed(kx + ky)
    X = torch.randn((kx, N), generator=g, dtype=torch.float64, device="cuda")
    Cm = rng.standard_normal((kx, ky))
    ref = (torch.as_tensor(Cm.T, device="cuda") @ X)                    # ky x N
    scale = torch.linalg.norm(X, dim=0)[None, :] * float(np.linalg.norm(Cm, axis=0).max())
    for path, tol in ((0, 1e-15), (1, 1e-13)):
        Y = _run(torch, path, X, Cm)
        err = float(torch.max(torch.abs(Y - ref) / scale))
        assert err < tol, (path, err)
