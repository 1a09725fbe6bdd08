"""Matrix-free time evolution on the GPU (kf_drive_apply, kf_to_lab; kfgpu.timeevolve) against the
oracle's restatement (oracle/timeevolve.py) of the reference's drive Hamiltonian on a node's product
basis (src/quantumtoolbox.jl:84-99, basis = :free) and its to_lab (:25-37): the action of H(t) and of
the interaction-frame H_I(t) on complex blocks (host and device buffers), to_lab's known answers,
fixed-step evolutions against the oracle's same stepping, and the properties of the reference's tests
(test/quantumtoolbox/test_quantumtoolbox.jl): a block evolves as its kets, the interaction frame
taken back to the lab frame equals the lab frame, no drives give e^{-i 2 pi (H0 - E0) T}.
Tolerances: one application 1e-12 of the result's scale (FP64, a different summation order);
evolutions against the oracle's same RK4 1e-10; the physics properties 1e-7, as the reference's tests.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import timeevolve as ote

pytestmark = pytest.mark.gpu


def _setup(ncut=4):
    from kfgpu import KronFreeOperator
    from test_timeevolve_oracle import system
    dims, terms, const, ports, H0d, Pd, E, V = system(ncut)
    H0 = KronFreeOperator(dims, terms, constant=const)
    Ps = [KronFreeOperator(dims, p) for p in ports]
    return H0, Ps, H0d, Pd, E, V


def _rand_block(N, m, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((N, m)) + 1j * rng.standard_normal((N, m))


@pytest.mark.parametrize("frame", ["lab", "interaction"])
def test_drive_apply_matches_oracle(cuda, frame):
    torch = cuda
    from kfgpu import timeevolve as te
    H0, Ps, H0d, Pd, E, V = _setup()
    funcs = [lambda t: 0.05 * math.cos(3.0 * t), lambda t: -0.02 + 0.01 * t]
    H = te.DriveHamiltonian(H0, list(zip(Ps, funcs)), E[0], frame=frame)
    om = ote.omega_of(H0d, E[0]) if frame == "interaction" else None
    if om is not None:
        assert np.allclose(H.omega, om, rtol=1e-13, atol=1e-12)
    X = _rand_block(H0.N, 3, 1)
    for t in (0.0, 0.37, 2.5):
        ref = ote.apply(H0d, E[0], Pd, funcs, t, X, omega=om)
        scale = np.max(np.abs(ref))
        got = H.apply(t, X)                                   # host buffers
        assert np.max(np.abs(got - ref)) / scale < 1e-12, (frame, t)
        P = te._pack(torch.as_tensor(X.T.copy(), device="cuda"))   # device buffers
        Y = H.apply_device(t, P)
        torch.cuda.synchronize()
        gd = (Y[:3] + 1j * Y[3:]).cpu().numpy().T
        assert np.max(np.abs(gd - ref)) / scale < 1e-12, (frame, t)
    # a single ket
    x = X[:, 1]
    assert np.max(np.abs(H.apply(0.37, x) - ote.apply(H0d, E[0], Pd, funcs, 0.37, x, omega=om))) < 1e-12 * scale


def test_to_lab_known_answers_and_oracle(cuda):
    torch = cuda
    from kfgpu import timeevolve as te
    psi = np.array([1.0, 2.0])
    assert te.to_lab(None, psi, 3.0) is psi
    assert np.allclose(te.to_lab([0.0, 1.0], np.array([1.0, 1.0]), math.pi), [1, -1])
    assert np.allclose(te.to_lab([0.0, 1.0], np.array([[1.0, 2.0], [1.0, 2.0]]), math.pi), [[1, 2], [-1, -2]])
    rng = np.random.default_rng(3)
    om = rng.uniform(-50, 50, 1000)
    X = _rand_block(1000, 4, 2)
    ref = ote.to_lab(om, X, 0.73)
    assert np.max(np.abs(te.to_lab(om, X, 0.73) - ref)) < 1e-12
    Xd = torch.as_tensor(X.T.copy(), device="cuda")
    got = te.to_lab(om, Xd, 0.73).cpu().numpy().T
    assert np.max(np.abs(got - ref)) < 1e-12
    from kfgpu import _abi
    with pytest.raises(_abi.DimensionMismatch, match="frequencies"):
        te.to_lab(om[:10], X, 1.0)


def test_sesolve_matches_oracle_stepping(cuda):
    from kfgpu import timeevolve as te
    H0, Ps, H0d, Pd, E, V = _setup()
    wd = 2 * math.pi * (E[1] - E[0])
    funcs = [lambda t: 0.05 * math.cos(wd * t)]
    H = te.DriveHamiltonian(H0, list(zip(Ps[:1], funcs)), E[0])
    psi0 = (V[:, 0] + 0.6 * V[:, 1]).astype(np.complex128)
    psi0 /= np.linalg.norm(psi0)
    tl = [0.0, 0.05, 0.1]
    got = te.sesolve(H, psi0, tl, 2e-3)
    ref = ote.rk4(H0d, E[0], Pd[:1], funcs, psi0, tl, 2e-3)
    assert got.shape == ref.shape == (3, H0.N)
    assert np.max(np.abs(got - ref)) < 1e-10


def test_block_evolves_as_its_kets_and_frames_agree(cuda):
    from kfgpu import timeevolve as te
    H0, Ps, H0d, Pd, E, V = _setup()
    wd = 2 * math.pi * (E[1] - E[0])
    drives = [(Ps[0], lambda t: 0.05 * math.cos(wd * t)), (Ps[1], lambda t: 0.02 * math.sin(0.5 * wd * t))]
    Hl = te.DriveHamiltonian(H0, drives, E[0])
    Hi = te.DriveHamiltonian(H0, drives, E[0], frame="interaction")
    B0 = np.stack([V[:, 0], (V[:, 1] + V[:, 2]) / math.sqrt(2), V[:, 3]], axis=1).astype(np.complex128)
    T, dt = 0.3, 1e-4
    Bl = te.sesolve(Hl, B0, [0.0, T], dt)[-1]
    for j in range(3):
        assert np.max(np.abs(te.sesolve(Hl, B0[:, j], [0.0, T], dt)[-1] - Bl[:, j])) < 1e-12
    Bi = te.sesolve(Hi, B0, [0.0, T], dt)[-1]
    assert np.max(np.abs(te.to_lab(Hi.omega, Bi, T) - Bl)) < 1e-7
    assert np.allclose(np.linalg.norm(Bl, axis=0), 1.0, atol=1e-9)


def test_no_drives_is_the_product_basis_propagator(cuda):
    from kfgpu import timeevolve as te
    H0, Ps, H0d, Pd, E, V = _setup()
    psi0 = (V[:, 0] + V[:, 1] + V[:, 4]).astype(np.complex128) / math.sqrt(3)
    T = 0.3
    got = te.sesolve(te.DriveHamiltonian(H0, [], E[0]), psi0, [0.0, T], 1e-4)[-1]
    assert np.max(np.abs(got - ote.expm_evolve(H0d, E[0], [], [], psi0, T))) < 1e-7


def test_drive_errors(cuda):
    from kfgpu import KronFreeOperator, _abi, timeevolve as te
    from kfgpu.ops import ChargeBasis, localop
    H0, Ps, H0d, Pd, E, V = _setup()
    small = KronFreeOperator([5], [(1.0, [(0, localop(ChargeBasis(2), "n"))])])
    with pytest.raises(_abi.DimensionMismatch):
        te.DriveHamiltonian(H0, [(small, lambda t: 1.0)], E[0])
    with pytest.raises(_abi.ArgumentError, match="frame"):
        te.DriveHamiltonian(H0, [], E[0], frame="bogus")
    # the library's own checks: a port on another basis, FP32
    X = np.zeros((H0.N, 2), order="F")
    ports = (C.c_void_p * 1)(small.handle)
    coef = (C.c_double * 1)(1.0)
    st = _abi.lib().kf_drive_apply(H0.handle, 0.0, 1, C.cast(ports, C.c_void_p), None, C.cast(coef, C.c_void_p), None,
                                   0.0, X.ctypes.data_as(C.c_void_p), H0.N, X.ctypes.data_as(C.c_void_p), H0.N, 1,
                                   _abi.KF_HOST | _abi.KF_F64)
    assert st == _abi.KF_EDIM
    st = _abi.lib().kf_drive_apply(H0.handle, 0.0, 0, None, None, None, None, 0.0, X.ctypes.data_as(C.c_void_p), H0.N,
                                   X.ctypes.data_as(C.c_void_p), H0.N, 1, _abi.KF_HOST | _abi.KF_F32)
    assert st == _abi.KF_EINVAL
    with pytest.raises(_abi.ArgumentError, match="neither"):
        te.DriveHamiltonian(H0, [((None, None), lambda t: 1.0)], E[0])


def _complex_ports(ncut=4):
    """e^{2 pi i n k} on mode 1 (k = 0.1: a port of complex character on the charge basis, as the
    reference's tests drive the real system) as (cos, sin) components, and an imaginary-only port."""
    from kfgpu import KronFreeOperator
    from kfgpu.ops import DiagonalOp
    n = np.arange(-ncut, ncut + 1, dtype=np.float64)
    d = 2 * ncut + 1
    c, sn = np.cos(2 * np.pi * 0.1 * n), np.sin(2 * np.pi * 0.1 * n)
    re = KronFreeOperator([d, d], [(1.0, [(0, DiagonalOp(c))])])
    im = KronFreeOperator([d, d], [(1.0, [(0, DiagonalOp(sn))])])
    im2 = KronFreeOperator([d, d], [(1.0, [(1, DiagonalOp(n))])])
    dense = np.kron(np.eye(d), np.diag(c + 1j * sn))          # axis 0 fastest
    dense2 = 1j * np.kron(np.diag(n), np.eye(d))
    return (re, im), (None, im2), dense, dense2


@pytest.mark.parametrize("frame", ["lab", "interaction"])
def test_complex_character_ports(cuda, frame):
    from kfgpu import timeevolve as te
    H0, Ps, H0d, Pd, E, V = _setup()
    p1, p2, d1, d2 = _complex_ports()
    funcs = [lambda t: 0.05 * math.cos(3.0 * t), lambda t: 0.02 * math.sin(2.0 * t)]
    H = te.DriveHamiltonian(H0, [(p1, funcs[0]), (p2, funcs[1])], E[0], frame=frame)
    om = ote.omega_of(H0d, E[0]) if frame == "interaction" else None
    X = _rand_block(H0.N, 2, 5)
    for t in (0.1, 1.3):
        ref = ote.apply(H0d, E[0], [d1, d2], funcs, t, X, omega=om)
        assert np.max(np.abs(H.apply(t, X) - ref)) / np.max(np.abs(ref)) < 1e-12, (frame, t)
    psi0 = (V[:, 0] + 0.5j * V[:, 1]).astype(np.complex128)
    got = te.sesolve(H, psi0, [0.0, 0.02, 0.04], 2e-3)
    ref = ote.rk4(H0d, E[0], [d1, d2], funcs, psi0, [0.0, 0.02, 0.04], 2e-3, omega=om)
    assert np.max(np.abs(got - ref)) < 1e-10
