"""The tensor-core FP32 Gram (tcgen05, TF32 hi / lo operands, FP32 accumulation in TMEM, FP64 sum
across CTAs) against a plain PyTorch FP64 product of the same FP32 data: the pools the LOBPCG loops
build -- [X Z]'Z of the orthogonalisation, [X_a Q]'[HX_a HZ] of the merged Rayleigh-Ritz Gram, the
refinement's [X_a R Q]'[R Q HZ] -- at block 16 and 20, self Grams, ragged widths, N not a multiple
of the 32-row chunk (zero-filled tail copies), a leading dimension above N, disjoint row and column
sources of up to 64 rows each (one MMA per K step on [A_hi; A_lo] x [B_hi; B_lo]), and the shapes
the kernel turns down (the solvers then keep the SIMT Gram).

The default kernel loads with 2-D tensor copies (128 rows x k columns per source); the cp.async
kernel, used where the CUDA driver gives no tensor-map encoder, runs the same pools in a subprocess with
KF_GRAM_TMA=0.

Tolerance: hi*hi + hi*lo + lo*hi drops lo*lo (2^-20 of a product) and TF32 keeps 10 mantissa bits
of lo (2^-21): 2e-6 of sqrt(sum|a|^2 sum|b|^2) per entry, as for the SIMT FP32 Gram.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(blocks, r0, r1, c0, c1, N, reps=1):
    """blocks: torch (k x ld) FP32 tensors = column-major N x k blocks, leading dimension ld."""
    from kfgpu import _abi
    ns = len(blocks)
    ptrs = (C.c_void_p * ns)(*[b.data_ptr() for b in blocks])
    lds = (C.c_int64 * ns)(*[b.stride(0) for b in blocks])
    ks = (C.c_int32 * ns)(*[b.shape[0] for b in blocks])
    nr = sum(b.shape[0] for b in blocks[r0:r1])
    nc = sum(b.shape[0] for b in blocks[c0:c1])
    G = np.zeros(nr * nc)
    ms = C.c_float(0)
    st = _abi.lib().kf_test_gram_tc(C.cast(ptrs, C.c_void_p), C.cast(lds, C.c_void_p), C.cast(ks, C.c_void_p), ns,
                                    r0, r1, c0, c1, N, reps, None, C.byref(ms), G.ctypes.data_as(C.c_void_p))
    return st, G.reshape(nc, nr).T, ms.value


def _check(torch, blocks, r0, r1, c0, c1, N):
    from kfgpu import _abi
    st, G, _ = _run(blocks, r0, r1, c0, c1, N)
    _abi.check(st)
    R = torch.cat([b[:, :N] for b in blocks[r0:r1]]).double()
    Q = torch.cat([b[:, :N] for b in blocks[c0:c1]]).double()
    ref = (R @ Q.T).cpu().numpy()
    scale = np.sqrt(np.outer((R ** 2).sum(1).cpu().numpy(), (Q ** 2).sum(1).cpu().numpy()))
    err = np.max(np.abs(G - ref) / scale)
    assert np.all(np.isfinite(G)) and err < 2e-6, err


def _blocks(torch, widths, N, ld=None, seed=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    ld = ld or N
    return [torch.randn(k, ld, generator=g, device="cuda", dtype=torch.float32) for k in widths]


POOLS = [
    # (widths, r0, r1, c0, c1, N); the pools up to 64 rows (sources in 8-row groups) take one MMA per
    # K step, the others two
    ((16, 32), 0, 2, 1, 2, 671744),              # [X Z]'Z, block 16 (64-row pool)
    ((20, 40), 0, 2, 1, 2, 671744),              # [X Z]'Z, block 20 (24 + 40 rows: one MMA)
    ((20, 44), 0, 2, 1, 2, 131072),              # 24 + 48 rows: two MMAs per K step
    ((16, 32, 16, 32), 0, 2, 2, 4, 671744),      # [X_a Q]'[HX_a HZ]
    ((20, 40, 20, 40), 0, 2, 2, 4, 671744),      # also the refinement's [X_a Q]'[R HZ]
    ((8, 16, 24), 0, 2, 1, 3, 131072),           # a source both in the rows and the columns
    ((16,), 0, 1, 0, 1, 671744),                 # self Gram
    ((32, 32), 0, 2, 0, 2, 110592),              # self Gram of 64 columns
    ((7, 13), 0, 2, 1, 2, 100000),
    ((1, 3), 0, 1, 1, 2, 5000),
    ((3, 5, 2, 9), 1, 3, 2, 4, 131072),          # a source in neither range
    ((12, 24), 0, 2, 1, 2, 33),                  # two chunks, the second one row long
    # disjoint row and column sources over 64 rows together: the one-MMA split layout
    ((7, 13, 30, 2), 0, 2, 2, 4, 131072),
    ((40, 24), 0, 1, 1, 2, 671744),
    ((64, 64), 0, 1, 1, 2, 100000),              # 64 + 64 rows, the largest split pool
    ((24, 40), 1, 2, 0, 1, 99999 + 1),           # the column source listed first
    ((18, 36, 18, 36), 0, 2, 2, 4, 100003),      # the solver's block 18, ragged N
]


@pytest.mark.parametrize("widths,r0,r1,c0,c1,N", POOLS)
def test_gram_tc_against_fp64(cuda, widths, r0, r1, c0, c1, N):
    torch = cuda
    ld = (N + 3) // 4 * 4   # 16-byte copies: the leading dimension a multiple of 4
    _check(torch, _blocks(torch, widths, N, ld=ld, seed=sum(widths) + N % 97), r0, r1, c0, c1, N)


@pytest.mark.parametrize("N", [100001, 100002, 100003, 4099])
def test_gram_tc_ragged_rows(cuda, N):
    """N not a multiple of 4 or of the chunk: the last copies are partly or wholly zero-filled."""
    torch = cuda
    ld = (N + 3) // 4 * 4 + 8
    _check(torch, _blocks(torch, (16, 32), N, ld=ld, seed=N), 0, 2, 1, 2, N)


def test_gram_tc_rejects_unfit_shapes(cuda):
    torch = cuda
    from kfgpu import _abi
    N = 4096
    # column sources over 64 columns
    st, _, _ = _run(_blocks(torch, (8, 72), N), 0, 2, 1, 2, N)
    assert st == _abi.KF_EINVAL
    # row-only and column sources over 128 rows
    st, _, _ = _run(_blocks(torch, (64, 64, 8), N), 0, 3, 0, 1, N)
    assert st == _abi.KF_EINVAL
    # leading dimension not a multiple of 4 (16-byte copies)
    st, _, _ = _run(_blocks(torch, (8, 8), N, ld=N + 1), 0, 2, 1, 2, N)
    assert st == _abi.KF_EINVAL


def test_gram_tc_repeated_launches_agree(cuda):
    """Deterministic: the FP32 partials are summed in a fixed order."""
    torch = cuda
    from kfgpu import _abi
    blocks = _blocks(torch, (16, 32), 671744, seed=11)
    st1, G1, _ = _run(blocks, 0, 2, 1, 2, 671744, reps=3)
    st2, G2, _ = _run(blocks, 0, 2, 1, 2, 671744, reps=1)
    _abi.check(st1)
    _abi.check(st2)
    assert np.array_equal(G1, G2)


def test_gram_tc_cp_async_kernel(cuda):
    """The pools and ragged row counts above on the cp.async kernel (KF_GRAM_TMA=0 at start-up)."""
    if os.environ.get("KF_GRAM_TMA") == "0":
        pytest.skip("this is the cp.async run")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-p", "no:cacheprovider", os.path.abspath(__file__),
                        "-k", "against_fp64 or ragged or repeated"],
                       env={**os.environ, "KF_GRAM_TMA": "0"}, capture_output=True, text=True, cwd=root)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert " passed" in r.stdout
