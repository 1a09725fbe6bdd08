"""The host symmetric eigensolver behind the Rayleigh-Ritz, SVQB and per-axis eigenbasis steps
(Householder tridiagonalisation + implicit QR with Wilkinson shifts) against numpy.linalg.eigh, through
the C ABI's host-only test entry (no GPU): random, graded, banded finite-difference, degenerate,
diagonal, zero and tiny matrices, a leading dimension above n, and unsymmetric input (the average of
the two triangles is what is solved, as the reference's Hermitian(...) wrappers do).

From n = 128 the eigenvectors are built by independent row blocks on several host threads (the
sizes 129 and 200 leave a short last block).

Tolerances: eigenvalues within 1e-13 ||A|| of LAPACK's; ||A V - V diag(w)|| <= 1e-13 n ||A||;
||V'V - I|| <= 1e-13 n.
"""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from kfgpu.build import build_library
    build_library()
    from kfgpu import _abi
    return _abi


def _eig(abi, A, lda=None):
    n = A.shape[0]
    lda = lda or n
    Ab = np.zeros((lda, n), order="F")
    Ab[:n, :n] = A
    Af = np.asfortranarray(Ab)
    w = np.zeros(n)
    V = np.zeros((n, n), order="F")
    abi.check(abi.lib().kf_test_sym_eig(n, Af.ctypes.data_as(C.c_void_p), lda, w.ctypes.data_as(C.c_void_p),
                                        V.ctypes.data_as(C.c_void_p), n))
    return w, V


def _check(abi, A, lda=None):
    n = A.shape[0]
    S = 0.5 * (A + A.T)
    w, V = _eig(abi, A, lda)
    nrm = max(np.linalg.norm(S, 2), 1e-300)
    wr = np.linalg.eigvalsh(S)
    assert np.all(np.diff(w) >= 0)
    assert np.max(np.abs(w - wr)) <= 1e-13 * nrm + 1e-300
    assert np.linalg.norm(S @ V - V * w) <= 1e-13 * n * nrm + 1e-300
    assert np.max(np.abs(V.T @ V - np.eye(n))) <= 1e-13 * max(n, 4)


def _fd(n, h=0.1):
    """A graded finite-difference operator: -d2/dx2 (5-point) + x^2 on n points."""
    c = np.array([-1 / 12, 4 / 3, -5 / 2, 4 / 3, -1 / 12]) / h ** 2
    A = np.zeros((n, n))
    for o, v in zip(range(-2, 3), c):
        A -= np.diag(np.full(n - abs(o), v), o)
    x = (np.arange(n) - n / 2) * h
    return A + np.diag(x ** 2)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 7, 18, 41, 54, 64, 127, 128, 129, 200, 256])
def test_random_symmetric(lib, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    _check(lib, A + A.T)


@pytest.mark.parametrize("n", [41, 64, 256])
def test_banded_finite_difference(lib, n):
    _check(lib, _fd(n))


def test_degenerate_and_structured(lib):
    rng = np.random.default_rng(3)
    n = 54
    Q = np.linalg.qr(rng.standard_normal((n, n)))[0]
    lam = np.repeat([-2.0, 0.0, 1.0, 5.0], [10, 20, 4, 20]) + np.concatenate([np.zeros(50), 1e-12 * np.arange(4)])
    _check(lib, (Q * lam) @ Q.T)                        # repeated eigenvalues
    _check(lib, np.diag(rng.standard_normal(n)))         # already diagonal
    _check(lib, np.zeros((n, n)))                        # zero matrix
    _check(lib, np.eye(n))                               # identity
    _check(lib, -np.diag(np.geomspace(1, 1e12, n)))      # graded, negative definite
    B = rng.standard_normal((n, n))
    _check(lib, B)                                       # unsymmetric: the triangles' average


def test_leading_dimension_above_n(lib):
    rng = np.random.default_rng(5)
    A = rng.standard_normal((20, 20))
    _check(lib, A + A.T, lda=27)


def test_rejects_bad_arguments(lib):
    from kfgpu._abi import ArgumentError
    w = np.zeros(4)
    V = np.zeros(16)
    A = np.zeros(16)
    with pytest.raises(ArgumentError):
        lib.check(lib.lib().kf_test_sym_eig(4, A.ctypes.data_as(C.c_void_p), 3, w.ctypes.data_as(C.c_void_p),
                                            V.ctypes.data_as(C.c_void_p), 4))
