"""kf_op_apply_noalloc, the operator application for callers that must not allocate device memory.

Such a caller (one whose device memory belongs to its own pool or arena, or a solver loop that
cannot take a cudaMalloc's synchronisation) gets the same Y = H X as kf_op_apply, with the
scratch of the dense-factor chains taken from one fixed static device array instead of a
cudaMalloc.  Checked here through the C ABI against kf_op_apply on an operator whose terms have
dense factors (so the scratch is used), twice in a row (the array keeps the previous call's
contents), in FP64 (to 1e-12 relative) and FP32 (to 2e-6 relative), and the rejection of a block
too wide for the fixed array.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _parent_op(d=12, seed=4):
    from kfgpu import KronFreeOperator, circuits
    dims, terms = circuits.dense_parent(np.random.default_rng(seed), d=d)
    return KronFreeOperator(dims, terms, block_capacity=16)


@pytest.mark.parametrize("f32,tol", [(False, 1e-12), (True, 2e-6)])
def test_noalloc_matches_apply_twice(cuda, f32, tol):
    torch = cuda
    from kfgpu import _abi
    L = _abi.lib()
    H = _parent_op()
    dt = torch.float32 if f32 else torch.float64
    flags = _abi.KF_F32 if f32 else _abi.KF_F64
    b = 16
    for call in range(2):
        X = torch.randn(b, H.N, dtype=dt, device="cuda", generator=torch.Generator("cuda").manual_seed(call))
        Y_ref = torch.empty_like(X)
        Y = torch.full_like(X, float("nan"))
        _abi.check(L.kf_op_apply(H.handle, X.data_ptr(), Y_ref.data_ptr(), H.N, H.N, b, flags))
        _abi.check(L.kf_op_apply_noalloc(H.handle, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), H.N, H.N, b,
                                         flags))
        H.sync()
        err = (Y - Y_ref).abs().max().item() / max(Y_ref.abs().max().item(), 1.0)
        assert err < tol, (call, err)


def test_noalloc_rejects_blocks_beyond_the_fixed_scratch(cuda):
    torch = cuda
    from kfgpu import _abi
    L = _abi.lib()
    H = _parent_op(d=16)                     # N = 4096; 2 N b doubles exceed 8 MiB from b = 129
    b = 160
    X = torch.zeros(b, H.N, dtype=torch.float64, device="cuda")
    Y = torch.zeros_like(X)
    st = L.kf_op_apply_noalloc(H.handle, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), H.N, H.N, b,
                               _abi.KF_F64)
    assert st == _abi.KF_EINVAL
    assert "KF_NOALLOC_SCRATCH_BYTES" in _abi.last_error()
