"""NumPy restatement of the reference's matrix-free time-evolution conventions (test infrastructure
only): the drive Hamiltonian on a node's product basis and the frame rotation.

  src/quantumtoolbox.jl:1-12    units and conventions: H/hbar = 2 pi [H0 - E0 + sum_k f_k(t) O_k]
                                (rad/ns, t in ns, f_k in GHz); batch = true evolves an N x m block
  src/quantumtoolbox.jl:25-37   to_lab: psi_lab = e^{-i Omega t} psi_I (rows rotated by their Omega)
  src/quantumtoolbox.jl:84-99   drive_hamiltonian: frame = :interaction is
                                H_I(t) = e^{i Omega t} (H(t) - diag Omega) e^{-i Omega t}, Omega the
                                diagonal of 2 pi (H0 - E0) in the evolved basis (matrix-free: its
                                diagonal entries)

The reference hands H(t) to QuantumToolbox's adaptive sesolve; `rk4` here is the same fixed-step
fourth-order Runge-Kutta as kfgpu.timeevolve.sesolve, so the two agree to rounding, and `expm_evolve`
(constant H) checks both against the exact propagator.
"""
from __future__ import annotations

import math

import numpy as np

TWO_PI = 2.0 * math.pi


def drive_matrix(H0, E0, ports, coefs):
    """2 pi [H0 - E0 + sum_k coefs[k] ports[k]] as a dense matrix (src/quantumtoolbox.jl:84-99); a port
    of complex character is a complex matrix."""
    M = np.array(H0, dtype=np.complex128) - E0 * np.eye(H0.shape[0])
    for O, c in zip(ports, coefs):
        M = M + c * np.asarray(O, dtype=np.complex128)
    return TWO_PI * M


def omega_of(H0, E0):
    """The interaction frame's Omega: the diagonal of 2 pi (H0 - E0) (src/quantumtoolbox.jl:84-99)."""
    return TWO_PI * (np.diag(H0) - E0)


def to_lab(omega, psi, t):
    """e^{-i Omega t} psi, rows rotated by their Omega; omega None: psi itself (src/quantumtoolbox.jl:25-37)."""
    if omega is None:
        return psi
    psi = np.asarray(psi)
    if psi.shape[0] != len(omega):
        raise ValueError(f"to_lab: the frame has {len(omega)} frequencies, the state {psi.shape[0]} rows")
    rot = np.exp(-1j * np.asarray(omega) * t)
    return rot[:, None] * psi if psi.ndim == 2 else rot * psi


def apply(H0, E0, ports, funcs, t, psi, omega=None):
    """H(t) psi in the lab frame, or H_I(t) psi with the frame's omega (src/quantumtoolbox.jl:84-99)."""
    M = drive_matrix(H0, E0, ports, [f(t) for f in funcs])
    if omega is None:
        return M @ psi
    rot = np.exp(-1j * omega * t)
    u = rot[:, None] * psi if psi.ndim == 2 else rot * psi
    y = M @ u - (omega[:, None] * u if psi.ndim == 2 else omega * u)
    return np.conj(rot)[:, None] * y if psi.ndim == 2 else np.conj(rot) * y


def rk4(H0, E0, ports, funcs, psi0, tlist, dt, omega=None):
    """States of d psi / dt = -i H(t) psi at tlist, RK4 with steps of at most dt (the stepping of
    kfgpu.timeevolve.sesolve)."""
    P = np.array(psi0, dtype=np.complex128)
    f = lambda t, x: -1j * apply(H0, E0, ports, funcs, t, x, omega)
    out = [P.copy()]
    t = float(tlist[0])
    for t1 in tlist[1:]:
        n = max(1, int(math.ceil((float(t1) - t) / dt - 1e-12)))
        h = (float(t1) - t) / n
        for _ in range(n):
            k1 = f(t, P)
            k2 = f(t + h / 2, P + (h / 2) * k1)
            k3 = f(t + h / 2, P + (h / 2) * k2)
            k4 = f(t + h, P + h * k3)
            P = P + (h / 6) * (k1 + 2 * k2 + 2 * k3 + k4)
            t += h
        t = float(t1)
        out.append(P.copy())
    return np.stack(out)


def expm_evolve(H0, E0, ports, coefs, psi0, T):
    """e^{-i H T} psi0 for constant coefficients (scipy's expm)."""
    from scipy.linalg import expm
    return expm(-1j * T * drive_matrix(H0, E0, ports, coefs)) @ psi0
