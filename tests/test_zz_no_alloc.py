"""kf_op_apply_noalloc, the operator application for callers that must not allocate device memory.

Such a caller owns its device memory through its own pool or arena (Julia's or PyTorch's caching
allocator, a fixed arena), or runs a solver loop that cannot take a cudaMalloc's device
synchronisation.  The entry point gives the same Y = H X as kf_op_apply, with the scratch of the
dense-factor chains in one fixed static device array.  Checked here through the C ABI:

  * on a fresh operator (never applied by kf_op_apply), after one set-up call per device on a
    different operator, repeated calls change the device's free memory by nothing and leave the
    operator's own scratch unallocated;
  * two calls in a row, each against kf_op_apply on a twin operator (1e-12 relative in FP64, 2e-6
    in FP32, the apply tests' tolerances) and against the oracle's FP64 mul!;
  * a block too wide for the fixed array is rejected.

This file is collected last on purpose: a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _terms(d=12, seed=4):
    from kfgpu import circuits
    return circuits.dense_parent(np.random.default_rng(seed), d=d)


def _op(dims, terms):
    from kfgpu import KronFreeOperator
    return KronFreeOperator(dims, terms, block_capacity=16)


def _oracle(dims, terms):
    from oracle import kfref
    from kfgpu import ops as P
    conv = [(c, [(a, kfref.DenseOp(op.M) if isinstance(op, P.DenseOp) else kfref.DiagonalOp(op.d)) for a, op in fs])
            for c, fs in terms]
    return kfref.KronFreeOperator(dims, conv)


def _scratch_bytes(L, H):
    v = C.c_uint64()
    assert L.kf_test_op_scratch_bytes(H.handle, C.byref(v)) == 0
    return v.value


@pytest.mark.parametrize("f32,tol", [(False, 1e-12), (True, 2e-6)])
def test_noalloc_allocates_nothing_and_matches_apply(cuda, f32, tol):
    torch = cuda
    from kfgpu import _abi
    L = _abi.lib()
    dims, terms = _terms()
    dt = torch.float32 if f32 else torch.float64
    flags = _abi.KF_F32 if f32 else _abi.KF_F64
    b = 16
    # every tensor this test touches exists before memory is measured
    gen = torch.Generator("cuda").manual_seed(11)
    N = int(np.prod(dims))
    Xs = [torch.randn(b, N, dtype=dt, device="cuda", generator=gen) for _ in range(2)]
    Ys = [torch.full_like(Xs[0], float("nan")) for _ in range(2)]
    Yref = [torch.empty_like(Xs[0]) for _ in range(2)]
    # set-up, once per device, on another operator: the address lookup (b = 0) and one call that
    # loads the kernels this precision uses
    Hs = _op(dims, terms)
    _abi.check(L.kf_op_apply_noalloc(Hs.handle, C.c_void_p(Xs[0].data_ptr()), C.c_void_p(Ys[0].data_ptr()), N, N, 0,
                                     flags))
    _abi.check(L.kf_op_apply_noalloc(Hs.handle, C.c_void_p(Xs[0].data_ptr()), C.c_void_p(Ys[0].data_ptr()), N, N, b,
                                     flags))
    Hs.sync()
    # the fresh operator and its twin for kf_op_apply
    H = _op(dims, terms)
    Ht = _op(dims, terms)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for call in range(2):
        _abi.check(L.kf_op_apply_noalloc(H.handle, C.c_void_p(Xs[call].data_ptr()), C.c_void_p(Ys[call].data_ptr()),
                                         N, N, b, flags))
    H.sync()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0, "kf_op_apply_noalloc changed the device's free memory"
    assert _scratch_bytes(L, H) == 0
    # the same blocks through the allocating entry point (on the twin) and the oracle
    for call in range(2):
        _abi.check(L.kf_op_apply(Ht.handle, Xs[call].data_ptr(), Yref[call].data_ptr(), N, N, b, flags))
    Ht.sync()
    assert _scratch_bytes(L, Ht) > 0
    Ho = _oracle(dims, terms)
    for call in range(2):
        Y, Yr = Ys[call], Yref[call]
        err = (Y - Yr).abs().max().item() / max(Yr.abs().max().item(), 1.0)
        assert err < tol, (call, err)
        X64 = Xs[call].double().cpu().numpy().T
        Yo = Ho.matvec(np.asfortranarray(X64))
        erro = np.max(np.abs(Y.double().cpu().numpy().T - Yo)) / max(np.max(np.abs(Yo)), 1.0)
        assert erro < tol, (call, erro)


def test_noalloc_rejects_blocks_beyond_the_fixed_scratch(cuda):
    torch = cuda
    from kfgpu import _abi
    L = _abi.lib()
    dims, terms = _terms(d=16)               # N = 4096; 2 N b doubles exceed 8 MiB from b = 129
    H = _op(dims, terms)
    b = 160
    X = torch.zeros(b, H.N, dtype=torch.float64, device="cuda")
    Y = torch.zeros_like(X)
    st = L.kf_op_apply_noalloc(H.handle, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), H.N, H.N, b,
                               _abi.KF_F64)
    assert st == _abi.KF_EINVAL
    assert "KF_NOALLOC_SCRATCH_BYTES" in _abi.last_error()
