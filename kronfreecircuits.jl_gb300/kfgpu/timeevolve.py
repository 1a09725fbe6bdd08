"""Matrix-free time evolution under port drives, on the GPU (kf_drive_apply, kf_to_lab).

  DriveHamiltonian(H0, drives, E0, frame)   src/quantumtoolbox.jl:84-99   drive_hamiltonian, basis = :free
  to_lab(omega, psi, t)                     src/quantumtoolbox.jl:25-37
  sesolve(H, psi0, tlist, dt)               a fixed-step RK4 driver of H's action (the reference hands
                                            its QobjEvo to QuantumToolbox's adaptive sesolve)

H(t) = 2 pi [H0 - E0 + sum_k f_k(t) O_k] in rad/ns (t in ns, f_k in GHz, E0 the node's lowest
energy), for a real H0 and port operators O_k on the same product basis: a KronFreeOperator (a port
of real character) or a pair (O_re, O_im) of its real and imaginary components (complex character,
e^{i phi} or e^{2 pi i n k}; either may be None).
frame = "interaction": H_I(t) = e^{i Omega t} (H(t) - diag Omega) e^{-i Omega t} with Omega the
diagonal of 2 pi (H0 - E0); to_lab takes its states back to the lab frame.  States are complex
(N,) kets or (N, m) blocks; on the device they are torch complex128 tensors, shape (m, N).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi

TWO_PI = 2.0 * math.pi


def _pack(psi):
    """(m, N) complex128 torch tensor -> (2m, N) float64: real rows, then imaginary rows (column-major
    N x 2m blocks for the library)."""
    import torch
    return torch.cat([psi.real, psi.imag]).contiguous()


def _unpack(P, m):
    import torch
    return torch.complex(P[:m], P[m:])


class DriveHamiltonian:
    """The drive Hamiltonian of src/quantumtoolbox.jl:84-99 on a node's product basis.  drives: a list
    of (O_k, f_k) pairs, O_k a KronFreeOperator on H0's basis (a port operator) or a pair of its real
    and imaginary components, f_k(t) its coefficient in GHz.  frame: "lab" or "interaction"."""

    def __init__(self, H0, drives, E0, frame="lab"):
        if frame not in ("lab", "interaction"):
            raise _abi.ArgumentError(_abi.KF_EINVAL, f"drive_hamiltonian: frame must be lab or interaction, got {frame!r}")
        self.H0 = H0
        self.E0 = float(E0)
        self.ports, self.ports_im = [], []
        for O, _ in drives:
            re, im = (O if isinstance(O, tuple) else (O, None))
            self.ports.append(re)
            self.ports_im.append(im)
        self.funcs = [f for _, f in drives]
        for k, (re, im) in enumerate(zip(self.ports, self.ports_im)):
            if re is None and im is None:
                raise _abi.ArgumentError(_abi.KF_EINVAL, f"drive_hamiltonian: port {k} has neither component")
            for O in (re, im):
                if O is not None and O.N != H0.N:
                    raise _abi.DimensionMismatch(_abi.KF_EDIM, f"drive_hamiltonian: port operator {k} has size "
                                                               f"{O.N}, H0 {H0.N}")
        self.frame = frame
        self.omega = None
        self._omega_dev = None
        if frame == "interaction":
            self.omega = TWO_PI * (np.asarray(H0.diagonal(), dtype=np.float64) - self.E0)

    @property
    def N(self):
        return self.H0.N

    def _omega_device(self):
        import torch
        if self._omega_dev is None:
            self._omega_dev = torch.as_tensor(self.omega, dtype=torch.float64, device="cuda")
        return self._omega_dev

    def apply_device(self, t, P, Y=None):
        """Y = H(t) P for a packed device block P ((2m, N) float64, real rows then imaginary rows), on
        torch's current stream (H0's stream is set to it)."""
        import torch
        cs = torch.cuda.current_stream().cuda_stream
        if getattr(self, "_stream", None) != cs:
            self.H0.set_stream(cs)
            self._stream = cs
        m = P.shape[0] // 2
        if Y is None:
            Y = torch.empty_like(P)
        coef, ports, pim = self._args(t)
        om = self._omega_device().data_ptr() if self.omega is not None else None
        _abi.check(_abi.lib().kf_drive_apply(self.H0.handle, self.E0, len(self.ports), ports, pim, coef, om, float(t),
                                             P.data_ptr(), self.N, Y.data_ptr(), self.N, m,
                                             _abi.KF_DEVICE | _abi.KF_F64))
        return Y

    def _args(self, t):
        """(coefficients, real components, imaginary components) as C arrays for kf_drive_apply."""
        n = max(1, len(self.funcs))
        coef = (C.c_double * n)(*[float(f(t)) for f in self.funcs])
        re = (C.c_void_p * n)(*[O.handle if O is not None else None for O in self.ports])
        im = (C.c_void_p * n)(*[O.handle if O is not None else None for O in self.ports_im])
        has_im = any(O is not None for O in self.ports_im)
        return C.cast(coef, C.c_void_p), C.cast(re, C.c_void_p), (C.cast(im, C.c_void_p) if has_im else None)

    def apply(self, t, psi):
        """H(t) psi for a host complex ket (N,) or block (N, m)."""
        X = np.asarray(psi, dtype=np.complex128)
        one = X.ndim == 1
        X = X.reshape(self.N, -1)
        m = X.shape[1]
        P = np.asfortranarray(np.concatenate([X.real, X.imag], axis=1))
        Y = np.empty_like(P, order="F")
        coef, ports, pim = self._args(t)
        om = self.omega.ctypes.data_as(C.c_void_p) if self.omega is not None else None
        _abi.check(_abi.lib().kf_drive_apply(self.H0.handle, self.E0, len(self.ports), ports, pim, coef, om, float(t),
                                             P.ctypes.data_as(C.c_void_p), self.N, Y.ctypes.data_as(C.c_void_p),
                                             self.N, m, _abi.KF_HOST | _abi.KF_F64))
        out = Y[:, :m] + 1j * Y[:, m:]
        return out[:, 0] if one else out


def to_lab(omega, psi, t):
    """e^{-i Omega t} psi (src/quantumtoolbox.jl:25-37): psi a host ket (N,) or block (N, m), or a device
    complex128 tensor (m, N); omega None is the lab frame (psi itself)."""
    if omega is None:
        return psi
    om = np.asarray(omega, dtype=np.float64)
    if not isinstance(psi, np.ndarray) and hasattr(psi, "is_cuda"):
        import torch
        m, N = psi.shape
        if N != om.size:
            raise _abi.DimensionMismatch(_abi.KF_EDIM, f"to_lab: the frame has {om.size} frequencies, the state {N} rows")
        P = _pack(psi)
        w = torch.as_tensor(om, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _abi.check(_abi.lib().kf_to_lab(w.data_ptr(), N, float(t), P.data_ptr(), N, m, _abi.KF_DEVICE | _abi.KF_F64))
        return _unpack(P, m)
    X = np.asarray(psi, dtype=np.complex128)
    one = X.ndim == 1
    X = X.reshape(X.shape[0], -1)
    N, m = X.shape
    if N != om.size:
        raise _abi.DimensionMismatch(_abi.KF_EDIM, f"to_lab: the frame has {om.size} frequencies, the state {N} rows")
    P = np.asfortranarray(np.concatenate([X.real, X.imag], axis=1))
    _abi.check(_abi.lib().kf_to_lab(om.ctypes.data_as(C.c_void_p), N, float(t), P.ctypes.data_as(C.c_void_p), N, m,
                                    _abi.KF_HOST | _abi.KF_F64))
    out = P[:, :m] + 1j * P[:, m:]
    return out[:, 0] if one else out


def sesolve(H, psi0, tlist, dt):
    """States of d psi / dt = -i H(t) psi at the times of tlist (ns, increasing, tlist[0] the start),
    classic fourth-order Runge-Kutta with steps of at most dt, on the device.  psi0: host ket (N,) or
    block (N, m); returns host arrays (len(tlist), N) or (len(tlist), N, m)."""
    import torch
    X = np.asarray(psi0, dtype=np.complex128)
    one = X.ndim == 1
    X = X.reshape(H.N, -1)
    m = X.shape[1]
    P = torch.as_tensor(np.concatenate([X.real.T, X.imag.T]), dtype=torch.float64, device="cuda").contiguous()

    def rhs(t, Q):
        Y = H.apply_device(t, Q)          # H(t) Q; -i H(t) Q: real rows <- imag, imag rows <- -real
        return torch.cat([Y[m:], -Y[:m]])

    out = [P.clone()]
    t = float(tlist[0])
    for t1 in tlist[1:]:
        n = max(1, int(math.ceil((float(t1) - t) / dt - 1e-12)))
        h = (float(t1) - t) / n
        for _ in range(n):
            k1 = rhs(t, P)
            k2 = rhs(t + h / 2, P + (h / 2) * k1)
            k3 = rhs(t + h / 2, P + (h / 2) * k2)
            k4 = rhs(t + h, P + h * k3)
            P = P + (h / 6) * (k1 + 2 * k2 + 2 * k3 + k4)
            t += h
        t = float(t1)
        out.append(P.clone())
    H.H0.sync()
    res = np.stack([(Q[:m] + 1j * Q[m:]).cpu().numpy().T for Q in out])
    return res[:, :, 0] if one else res
