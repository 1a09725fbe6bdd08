"""The FP32 LOBPCG iteration's device-side pieces: the second orthogonalisation pass's Cholesky
coefficients (k_chol2_coeffs) against a NumPy restatement -- including the failure status that
sends the solver to the host SVQB pass -- and the pipelined update with its output split over two
blocks (the fused X_new / P_new Rayleigh-Ritz update) against a PyTorch FP64 product."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _chol2(G, wx, r):
    from kfgpu import _abi
    Gf = np.asfortranarray(G)
    Cout = np.zeros((r + wx) * r)
    st = C.c_int(-1)
    _abi.check(_abi.lib().kf_test_chol2(Gf.ctypes.data_as(C.c_void_p), wx, r, Cout.ctypes.data_as(C.c_void_p),
                                        C.byref(st)))
    return Cout.reshape(r, r + wx).T, st.value


@pytest.mark.parametrize("wx,r", [(18, 36), (16, 32), (0, 8), (20, 40), (3, 64)])
def test_chol2_orthonormalises(cuda, wx, r):
    """Z (FP64 stand-in for the FP32 block, N rows) nearly orthonormal after a first pass: the
    coefficients make [Z X] C orthonormal and orthogonal to X to FP32 accuracy."""
    rng = np.random.default_rng(wx * 100 + r)
    N = 4000
    X = np.linalg.qr(rng.standard_normal((N, wx)))[0] if wx else np.zeros((N, 0))
    Z = np.linalg.qr(rng.standard_normal((N, r)))[0] + 1e-3 * rng.standard_normal((N, r))
    Z -= X @ (X.T @ Z) * 0.99          # a first pass that left a little of X in Z
    G = np.vstack([X.T @ Z, Z.T @ Z])
    Cm, st = _chol2(G, wx, r)
    assert st == 0
    Q = np.hstack([Z, X]) @ Cm
    assert np.abs(Q.T @ Q - np.eye(r)).max() < 1e-5
    if wx:
        assert np.abs(X.T @ Q).max() < 1e-5


def test_chol2_reports_a_dependent_direction(cuda):
    rng = np.random.default_rng(7)
    N, r = 2000, 8
    Z = np.linalg.qr(rng.standard_normal((N, r)))[0]
    Z[:, 5] = Z[:, 2] + 1e-4 * Z[:, 6]   # nearly dependent: a pivot ~1e-8
    _, st = _chol2(np.asfortranarray(Z.T @ Z), 0, r)
    assert st == 1


@pytest.mark.parametrize("path", [0, 1])
@pytest.mark.parametrize("N,kx0,kx1,ky0,ky1", [(671744, 18, 36, 18, 18), (100000, 16, 32, 16, 16), (4096, 7, 5, 3, 9),
                                               (130000, 64, 0, 32, 32), (100003, 20, 40, 20, 20)])
def test_update_split_outputs(cuda, path, N, kx0, kx1, ky0, ky1):
    torch = cuda
    from kfgpu import _abi
    rng = np.random.default_rng(N + kx0)
    ld = (N + 3) // 4 * 4
    X0 = torch.as_tensor(rng.standard_normal((kx0, ld)), dtype=torch.float32, device="cuda")
    X1 = torch.as_tensor(rng.standard_normal((max(kx1, 1), ld)), dtype=torch.float32, device="cuda")
    Y0 = torch.as_tensor(rng.standard_normal((ky0, ld)), dtype=torch.float32, device="cuda")
    Y1 = torch.as_tensor(rng.standard_normal((max(ky1, 1), ld)), dtype=torch.float32, device="cuda")
    Cm = rng.standard_normal((kx0 + kx1, ky0 + ky1))
    Y0r, Y1r = Y0.clone(), Y1.clone()
    Cf = np.asfortranarray(Cm)
    _abi.check(_abi.lib().kf_test_update_split(path, C.c_void_p(Y0.data_ptr()), ky0, C.c_void_p(Y1.data_ptr()), ky1,
                                               C.c_void_p(X0.data_ptr()), kx0, C.c_void_p(X1.data_ptr()), kx1,
                                               Cf.ctypes.data_as(C.c_void_p), 0.5, 1.0, N, ld))
    Xa = torch.cat([X0[:, :N], X1[:kx1, :N]]).double()
    Ct = torch.as_tensor(Cm.astype(np.float32).astype(np.float64), device="cuda")
    ref = 0.5 * (Ct.T @ Xa)
    ref0 = ref[:ky0] + Y0r[:, :N].double()
    bound = 0.5 * (Ct.abs().T @ Xa.abs()) + 1.0
    assert ((Y0[:, :N].double() - ref0).abs() / bound[:ky0]).max().item() < 5e-6
    if ky1:
        ref1 = ref[ky0:] + Y1r[:ky1, :N].double()
        assert ((Y1[:ky1, :N].double() - ref1).abs() / bound[ky0:]).max().item() < 5e-6
