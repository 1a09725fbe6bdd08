"""Host-side local operators and single-mode bases, mirroring the reference's data model.

  src/localops.jl:11-73   DenseOp, DiagonalOp, BandedOp, ShiftOp (the four factor structures)
  src/bases.jl:113-239    ChargeBasis, PhaseGrid, PeriodicGrid and the ports they serve

The GPU path computes in real arithmetic (every measured circuit is real by structure), so
ports whose matrix is imaginary (-i d/dphi on a grid) or complex (e^{ik phi} on a grid) are
exposed through their real and imaginary components, the pieces the reference's real
expansion (src/character.jl:297-315) keeps: `localop(b, kind, k, part="re"|"im")`.
"""
from __future__ import annotations

import numpy as np

_FD1 = {2: [-1 / 2, 0, 1 / 2],
        4: [1 / 12, -2 / 3, 0, 2 / 3, -1 / 12],
        6: [-1 / 60, 3 / 20, -3 / 4, 0, 3 / 4, -3 / 20, 1 / 60],
        8: [1 / 280, -4 / 105, 1 / 5, -4 / 5, 0, 4 / 5, -1 / 5, 4 / 105, -1 / 280]}
_FD2 = {2: [1.0, -2.0, 1.0],
        4: [-1 / 12, 4 / 3, -5 / 2, 4 / 3, -1 / 12],
        6: [1 / 90, -3 / 20, 3 / 2, -49 / 18, 3 / 2, -3 / 20, 1 / 90],
        8: [-1 / 560, 8 / 315, -1 / 5, 8 / 5, -205 / 72, 8 / 5, -1 / 5, 8 / 315, -1 / 560]}


class DenseOp:
    kind = "dense"

    def __init__(self, M):
        M = np.asarray(M, dtype=np.float64)
        if M.ndim != 2 or M.shape[0] != M.shape[1]:
            raise ValueError(f"DenseOp requires a square matrix, got {M.shape}")
        self.M = np.asfortranarray(M)
        self.n = M.shape[0]

    def dense(self):
        return np.array(self.M)


class DiagonalOp:
    kind = "diag"

    def __init__(self, d):
        self.d = np.ascontiguousarray(d, dtype=np.float64)
        self.n = len(self.d)

    def dense(self):
        return np.diag(self.d)


class BandedOp:
    """Y[i] = sum_b weights[b][i] X[i + offsets[b]] over valid neighbours (src/localops.jl:40-41)."""

    kind = "banded"

    def __init__(self, n, offsets, weights):
        if len(offsets) != len(weights):
            raise ValueError("BandedOp: offsets and weights differ in length")
        self.n = int(n)
        self.offsets = [int(o) for o in offsets]
        self.weights = [np.asarray(w, dtype=np.float64) for w in weights]
        if any(len(w) != self.n for w in self.weights):
            raise ValueError("BandedOp: every weight vector must have length n")

    def dense(self):
        A = np.zeros((self.n, self.n))
        for o, w in zip(self.offsets, self.weights):
            for i in range(self.n):
                if 0 <= i + o < self.n:
                    A[i, i + o] += w[i]
        return A


class ShiftOp:
    """Y[i + s] = factor X[i] (src/localops.jl:61)."""

    kind = "shift"

    def __init__(self, n, s, factor=1.0):
        self.n, self.s, self.factor = int(n), int(s), float(factor)

    def dense(self):
        A = np.zeros((self.n, self.n))
        for i in range(self.n):
            if 0 <= i + self.s < self.n:
                A[i + self.s, i] = self.factor
        return A


class ChargeBasis:
    def __init__(self, ncut):
        if ncut < 0:
            raise ValueError("ChargeBasis requires ncut >= 0")
        self.ncut = int(ncut)
        self.dim = 2 * self.ncut + 1


class PhaseGrid:
    def __init__(self, a, b, N, order=8):
        if order not in (2, 4, 6, 8):
            raise ValueError("PhaseGrid order must be 2, 4, 6 or 8")
        if not b > a or not N > order:
            raise ValueError("PhaseGrid requires b > a and N > order")
        self.a, self.b, self.N, self.order = float(a), float(b), int(N), int(order)
        self.dim = self.N

    def coordinates(self):
        return np.linspace(self.a, self.b, self.N)

    def spacing(self):
        return (self.b - self.a) / (self.N - 1)


def localop(basis, kind, k=0.0, part="re"):
    """The real (`part="re"`) or imaginary (`part="im"`) component of port (kind, k) in `basis`."""
    if isinstance(basis, ChargeBasis):
        n = np.arange(-basis.ncut, basis.ncut + 1, dtype=np.float64)
        if kind in ("n", "n2"):
            return DiagonalOp(n if kind == "n" else n ** 2) if part == "re" else DiagonalOp(np.zeros(basis.dim))
        if kind == "expiphi":
            if abs(k - round(k)) > 1e-12:
                raise ValueError("ChargeBasis: expiphi needs an integer k")
            return ShiftOp(basis.dim, int(round(k)), 1.0 if part == "re" else 0.0)
    elif isinstance(basis, PhaseGrid):
        N, D, h = basis.N, basis.spacing(), basis.order // 2
        phi = basis.coordinates()
        if kind == "n":               # -i d/dphi: purely imaginary
            w = _FD1[basis.order]
            offs = [j for j in range(-h, h + 1) if j != 0]
            scale = 0.0 if part == "re" else 1.0
            return BandedOp(N, offs, [np.full(N, -scale * w[j + h] / D) for j in offs])
        if kind == "n2":              # -d^2/dphi^2
            w = _FD2[basis.order]
            scale = 1.0 if part == "re" else 0.0
            return BandedOp(N, list(range(-h, h + 1)), [np.full(N, -scale * w[j + h] / D ** 2) for j in range(-h, h + 1)])
        if kind == "phi":
            return DiagonalOp(phi if part == "re" else np.zeros(N))
        if kind == "phi2":
            return DiagonalOp(phi ** 2 if part == "re" else np.zeros(N))
        if kind == "expiphi":
            return DiagonalOp(np.cos(k * phi) if part == "re" else np.sin(k * phi))
    raise ValueError(f"{type(basis).__name__}: port {kind} is not available")
