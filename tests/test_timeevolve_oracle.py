"""The oracle's restatement of the reference's matrix-free time-evolution conventions
(oracle/timeevolve.py; src/quantumtoolbox.jl), pinned by the properties the reference's own tests
check (test/quantumtoolbox/test_quantumtoolbox.jl): to_lab's known answers on arrays (:102-107), the
interaction frame taken back to the lab frame equal to the lab-frame evolution, for a ket and for a
block (:109-128), and with no drives the product-basis evolution e^{-i 2 pi (H0 - E0) T} (:137-149);
and a Hermitian port of complex character keeps the evolution unitary.
The system: two transmons on the flat product of two small charge bases (9 x 9), driven through the
charge port of the first, f(t) = 0.05 cos(2 pi (E1 - E0) t) GHz, as the reference's tests drive.
"""
import math

import numpy as np
import pytest

from oracle import kfref, timeevolve as ote


def _dense(dims, terms, constant=0.0):
    from kfgpu import ops as P
    conv = []
    for c, fs in terms:
        g = []
        for a, op in fs:
            if isinstance(op, P.DiagonalOp):
                g.append((a, kfref.DiagonalOp(op.d)))
            elif isinstance(op, P.ShiftOp):
                g.append((a, kfref.ShiftOp(op.n, op.s, op.factor)))
            elif isinstance(op, P.BandedOp):
                g.append((a, kfref.BandedOp(op.n, op.offsets, op.weights)))
            else:
                g.append((a, kfref.DenseOp(op.dense())))
        conv.append((c, g))
    return kfref.KronFreeOperator(dims, conv, constant=constant).to_matrix().real


def system(ncut=4):
    """(dims, terms, constant, port terms, H0 dense, ports dense, E, V) of the test circuit."""
    from kfgpu import circuits
    from kfgpu.ops import ChargeBasis, localop
    th = {"E_J1": 9.0, "E_C1": 0.25, "n_g1": 0.1, "E_J2": 11.0, "E_C2": 0.22, "n_g2": 0.3, "g": 0.04}
    dims, terms, const = circuits.two_transmon_flat(th, ncut)
    b = ChargeBasis(ncut)
    ports = [[(1.0, [(0, localop(b, "n"))])],                                          # n on mode 1
             [(0.5, [(1, localop(b, "expiphi", 1))]), (0.5, [(1, localop(b, "expiphi", -1))])]]   # cos phi on mode 2
    H0 = _dense(dims, terms, const)
    Pd = [_dense(dims, p) for p in ports]
    E, V = np.linalg.eigh(H0)
    return dims, terms, const, ports, H0, Pd, E, V


def test_to_lab_known_answers():
    psi = np.array([1.0, 2.0])
    assert ote.to_lab(None, psi, 3.0) is psi
    assert np.allclose(ote.to_lab([0.0, 1.0], np.array([1.0, 1.0]), math.pi), [1, -1])
    assert np.allclose(ote.to_lab([0.0, 1.0], np.array([[1.0, 2.0], [1.0, 2.0]]), math.pi), [[1, 2], [-1, -2]])
    with pytest.raises(ValueError, match="frequencies"):
        ote.to_lab([0.0, 1.0, 2.0], np.array([1.0, 1.0]), 1.0)


def test_interaction_frame_back_to_lab():
    _, _, _, _, H0, Pd, E, V = system()
    wd = 2 * math.pi * (E[1] - E[0])
    funcs = [lambda t: 0.05 * math.cos(wd * t)]
    psi0 = (V[:, 0] + 0.6 * V[:, 1] - 0.3j * V[:, 2]).astype(np.complex128)
    psi0 /= np.linalg.norm(psi0)
    T, dt = 0.5, 1e-4
    om = ote.omega_of(H0, E[0])
    lab = ote.rk4(H0, E[0], Pd[:1], funcs, psi0, [0.0, T], dt)[-1]
    inter = ote.rk4(H0, E[0], Pd[:1], funcs, psi0, [0.0, T], dt, omega=om)[-1]
    assert np.max(np.abs(ote.to_lab(om, inter, T) - lab)) < 1e-7
    assert abs(np.linalg.norm(lab) - 1.0) < 1e-9
    # a block: each column as its own ket
    B0 = np.stack([psi0, V[:, 3].astype(np.complex128)], axis=1)
    Bl = ote.rk4(H0, E[0], Pd[:1], funcs, B0, [0.0, T], dt)[-1]
    assert np.max(np.abs(Bl[:, 0] - lab)) < 1e-13


def test_no_drives_is_the_product_basis_propagator():
    _, _, _, _, H0, Pd, E, V = system()
    psi0 = (V[:, 0] + V[:, 1] + V[:, 4]).astype(np.complex128) / math.sqrt(3)
    T = 0.5
    ex = ote.expm_evolve(H0, E[0], [], [], psi0, T)
    r = ote.rk4(H0, E[0], [], [], psi0, [0.0, T], 1e-4)[-1]
    assert np.max(np.abs(r - ex)) < 1e-7
    # dressed amplitudes pick up e^{-i 2 pi (E_i - E_0) T}
    amp = V.conj().T @ ex
    assert np.allclose(amp, np.exp(-1j * 2 * math.pi * (E - E[0]) * T) * (V.conj().T @ psi0), atol=1e-10)


def test_complex_character_port_is_unitary():
    """A Hermitian port of complex character -- the charge n = -i d/dphi on a phase grid, purely
    imaginary -- keeps the evolution unitary, and the fixed-step evolution matches e^{-i H T} for a
    constant coefficient."""
    from kfgpu import circuits
    from kfgpu.ops import PhaseGrid, localop
    rng = np.random.default_rng(9)
    dims, terms = circuits.fluxonium_leaf(circuits.fluxonium_theta(rng), 101)
    H0 = _dense(dims, terms)
    basis = PhaseGrid(-5 * math.pi, 5 * math.pi, 101, 4)        # the fluxonium leaf's grid
    n_im = _dense(dims, [(1.0, [(0, localop(basis, "n", part="im"))])])
    O = 1j * n_im
    assert np.allclose(O, O.conj().T, atol=1e-12)
    E = np.linalg.eigvalsh(H0)
    V = np.linalg.eigh(H0)[1]
    psi0 = (V[:, 0] + V[:, 1]).astype(np.complex128) / math.sqrt(2)
    T = 0.05
    ex = ote.expm_evolve(H0, E[0], [O], [0.03], psi0, T)
    r = ote.rk4(H0, E[0], [O], [lambda t: 0.03], psi0, [0.0, T], 1e-5)[-1]
    assert abs(np.linalg.norm(ex) - 1.0) < 1e-12
    assert np.max(np.abs(r - ex)) < 1e-7
