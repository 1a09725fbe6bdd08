"""NumPy restatement of the reference's operator layer (test infrastructure only).

Follows, file by file (paths within KronFreeCircuits.jl):
  src/localops.jl:11-188     DenseOp / DiagonalOp / BandedOp / ShiftOp, dense, diagonal, infnorm,
                             realpart / imagpart
  src/bases.jl:113-280       coordinates, spacing, finite-difference tables, localop per basis
  src/terms.jl:119-168       circuit_terms, constant_term
  src/parameters.jl:223-227  phase_factor
  src/character.jl:281-315   the real expansion Re(c ⊗ O) of a product term
  src/apply.jl:9-128         apply_axis! for every factor structure
  src/apply.jl:222-253       KronFreeOperator construction (all-diagonal terms fused into one diagonal)
  src/apply.jl:370-432       mul!: the fused diagonal, then one chained pass per kept term
  src/apply.jl:438-478       the diagonal of H
  src/apply.jl:506-531       Matrix(H) by applying H to identity blocks of <= 256 columns
  src/apply.jl:586-685       gershgorin_bound, separable_eigenbases, product_seed

Layout everywhere: column-major, axis 1 fastest, the block (column) axis last, as the
reference's `reshape(x, dims..., b)`.  Arrays here are NumPy arrays in Fortran order when
reshaped to the state tensor.
"""
from __future__ import annotations

import ast
import json
import math
from fractions import Fraction as F

import numpy as np

# --------------------------------------------------------------------------------------------
# Local operators (src/localops.jl)


class DenseOp:
    def __init__(self, M):
        M = np.asarray(M)
        if M.ndim != 2 or M.shape[0] != M.shape[1]:
            raise ValueError(f"DenseOp requires a square matrix, got {M.shape}")
        self.M = M.astype(np.complex128 if np.iscomplexobj(M) else np.float64)

    @property
    def n(self):
        return self.M.shape[0]

    def dense(self):
        return self.M.copy()

    def diagonal(self):
        return np.diag(self.M).copy()

    def infnorm(self):
        return float(np.max(np.sum(np.abs(self.M), axis=1))) if self.n else 0.0

    def realpart(self):
        return DenseOp(self.M.real.astype(np.float64))

    def imagpart(self):
        return DenseOp(np.imag(self.M).astype(np.float64))

    def adjoint(self):
        return DenseOp(self.M.conj().T.copy())


class DiagonalOp:
    def __init__(self, d):
        d = np.asarray(d)
        self.d = d.astype(np.complex128 if np.iscomplexobj(d) else np.float64)

    @property
    def n(self):
        return len(self.d)

    def dense(self):
        return np.diag(self.d)

    def diagonal(self):
        return self.d.copy()

    def infnorm(self):
        return float(np.max(np.abs(self.d))) if self.n else 0.0

    def realpart(self):
        return DiagonalOp(self.d.real.astype(np.float64))

    def imagpart(self):
        return DiagonalOp(np.imag(self.d).astype(np.float64))


class BandedOp:
    """Y[i] = sum_b weights[b][i] X[i + offsets[b]] over 1 <= i + offsets[b] <= n (src/localops.jl:40-41)."""

    def __init__(self, n, offsets, weights):
        if n < 0:
            raise ValueError("BandedOp requires n >= 0")
        if len(offsets) != len(weights):
            raise ValueError("BandedOp: offsets and weights differ in length")
        self.n = int(n)
        self.offsets = [int(o) for o in offsets]
        ws = [np.asarray(w) for w in weights]
        cplx = any(np.iscomplexobj(w) for w in ws)
        self.weights = [w.astype(np.complex128 if cplx else np.float64) for w in ws]
        for w in self.weights:
            if len(w) != self.n:
                raise ValueError("BandedOp: every weight vector must have length n")

    def dense(self):
        dt = self.weights[0].dtype if self.weights else np.float64
        A = np.zeros((self.n, self.n), dtype=dt)
        for o, w in zip(self.offsets, self.weights):
            for i in range(self.n):
                if 0 <= i + o < self.n:
                    A[i, i + o] += w[i]
        return A

    def diagonal(self):
        for o, w in zip(self.offsets, self.weights):
            if o == 0:
                return w.copy()
        return np.zeros(self.n)

    def infnorm(self):
        m = 0.0
        for i in range(self.n):
            r = 0.0
            for o, w in zip(self.offsets, self.weights):
                if 0 <= i + o < self.n:
                    r += abs(w[i])
            m = max(m, r)
        return float(m)

    def realpart(self):
        return BandedOp(self.n, list(self.offsets), [w.real.astype(np.float64) for w in self.weights])

    def imagpart(self):
        return BandedOp(self.n, list(self.offsets), [np.imag(w).astype(np.float64) for w in self.weights])


class ShiftOp:
    """Y[i + s] = factor X[i] for valid indices (src/localops.jl:61)."""

    def __init__(self, n, s, factor):
        if n < 0:
            raise ValueError("ShiftOp requires n >= 0")
        self.n, self.s, self.factor = int(n), int(s), factor

    def dense(self):
        A = np.zeros((self.n, self.n), dtype=np.result_type(self.factor, np.float64))
        for i in range(self.n):
            if 0 <= i + self.s < self.n:
                A[i + self.s, i] = self.factor
        return A

    def diagonal(self):
        return np.full(self.n, self.factor) if self.s == 0 else np.zeros(self.n)

    def infnorm(self):
        return float(abs(self.factor)) if abs(self.s) < self.n else 0.0

    def realpart(self):
        return ShiftOp(self.n, self.s, float(np.real(self.factor)))

    def imagpart(self):
        return ShiftOp(self.n, self.s, float(np.imag(self.factor)))


def is_zero_op(op):
    if isinstance(op, DenseOp):
        return not np.any(op.M)
    if isinstance(op, DiagonalOp):
        return not np.any(op.d)
    if isinstance(op, BandedOp):
        return not any(np.any(w) for w in op.weights)
    return op.factor == 0


# --------------------------------------------------------------------------------------------
# Bases (src/bases.jl:113-280)

_FD1 = {
    2: [F(-1, 2), F(0), F(1, 2)],
    4: [F(1, 12), F(-2, 3), F(0), F(2, 3), F(-1, 12)],
    6: [F(-1, 60), F(3, 20), F(-3, 4), F(0), F(3, 4), F(-3, 20), F(1, 60)],
    8: [F(1, 280), F(-4, 105), F(1, 5), F(-4, 5), F(0), F(4, 5), F(-1, 5), F(4, 105), F(-1, 280)],
}
_FD2 = {
    2: [F(1), F(-2), F(1)],
    4: [F(-1, 12), F(4, 3), F(-5, 2), F(4, 3), F(-1, 12)],
    6: [F(1, 90), F(-3, 20), F(3, 2), F(-49, 18), F(3, 2), F(-3, 20), F(1, 90)],
    8: [F(-1, 560), F(8, 315), F(-1, 5), F(8, 5), F(-205, 72), F(8, 5), F(-1, 5), F(8, 315), F(-1, 560)],
}


def fd_weights(order, derivative):
    """Central finite-difference weights (src/bases.jl:143-148)."""
    if order not in (2, 4, 6, 8):
        raise ValueError(f"fd_weights: order must be 2, 4, 6 or 8, got {order}")
    tab = {1: _FD1, 2: _FD2}.get(derivative)
    if tab is None:
        raise ValueError("fd_weights: derivative must be 1 or 2")
    return np.array([float(x) for x in tab[order]])


class ChargeBasis:
    kind = "c"

    def __init__(self, ncut):
        if ncut < 0:
            raise ValueError("ChargeBasis requires ncut >= 0")
        self.ncut = int(ncut)

    @property
    def dim(self):
        return 2 * self.ncut + 1


class PhaseGrid:
    kind = "e"

    def __init__(self, a, b, N, order=8):
        if order not in (2, 4, 6, 8):
            raise ValueError("PhaseGrid order must be 2, 4, 6 or 8")
        if not b > a:
            raise ValueError("PhaseGrid requires b > a")
        if not N > order:
            raise ValueError("PhaseGrid requires N > order")
        self.a, self.b, self.N, self.order = float(a), float(b), int(N), int(order)

    @property
    def dim(self):
        return self.N

    def coordinates(self):
        return np.linspace(self.a, self.b, self.N)

    def spacing(self):
        return (self.b - self.a) / (self.N - 1)


class PeriodicGrid:
    kind = "c"

    def __init__(self, N, order=8):
        if N < order + 1:
            raise ValueError("PeriodicGrid requires N >= order + 1")
        self.N, self.order = int(N), int(order)

    @property
    def dim(self):
        return self.N

    def coordinates(self):
        return -np.pi + 2 * np.pi * np.arange(self.N) / self.N

    def spacing(self):
        return 2 * np.pi / self.N


def _cyclic_stencil(N, h, c):
    """src/bases.jl:215-223."""
    offs, ws = [], []
    for j in range(-h, h + 1):
        if c[j + h] == 0:
            continue
        cand = (j, j + N) if j < 0 else (j, j - N) if j > 0 else (j,)
        for o in cand:
            offs.append(o)
            ws.append(np.array([c[j + h] if 0 <= i + o < N else 0 * c[j + h] for i in range(N)]))
    return BandedOp(N, offs, ws)


def localop(basis, kind, k=0.0):
    """The operator of port (kind, k) in `basis` (src/bases.jl:162-239)."""
    if isinstance(basis, ChargeBasis):
        n = np.arange(-basis.ncut, basis.ncut + 1, dtype=np.float64)
        d = basis.dim
        if kind == "n":
            return DiagonalOp(n)
        if kind == "n2":
            return DiagonalOp(n ** 2)
        if kind == "expiphi":
            if abs(k - round(k)) > 1e-12:
                raise ValueError("ChargeBasis: expiphi needs an integer k")
            return ShiftOp(d, int(round(k)), 1.0)
        if kind == "exp2pin":
            return DiagonalOp(np.exp(2j * np.pi * k * n))
    elif isinstance(basis, PhaseGrid):
        N, D, h = basis.N, basis.spacing(), basis.order // 2
        phi = basis.coordinates()
        if kind == "n":
            w = fd_weights(basis.order, 1)
            offs = [j for j in range(-h, h + 1) if j != 0]
            return BandedOp(N, offs, [np.full(N, -1j * w[j + h] / D) for j in offs])
        if kind == "n2":
            w = fd_weights(basis.order, 2)
            return BandedOp(N, list(range(-h, h + 1)), [np.full(N, -w[j + h] / D ** 2) for j in range(-h, h + 1)])
        if kind == "phi":
            return DiagonalOp(phi)
        if kind == "phi2":
            return DiagonalOp(phi ** 2)
        if kind == "expiphi":
            return DiagonalOp(np.exp(1j * k * phi))
        if kind == "exp2pin":
            s = 2 * np.pi * k / D
            if abs(s - round(s)) >= 1e-8:
                raise ValueError("PhaseGrid: exp2pin needs 2*pi*k/Delta integer")
            return ShiftOp(N, -int(round(s)), 1.0)
    elif isinstance(basis, PeriodicGrid):
        N, D, h = basis.N, basis.spacing(), basis.order // 2
        if kind == "n":
            return _cyclic_stencil(N, h, (-1j * fd_weights(basis.order, 1) / D).astype(np.complex128))
        if kind == "n2":
            return _cyclic_stencil(N, h, -fd_weights(basis.order, 2) / D ** 2)
        if kind == "expiphi":
            return DiagonalOp(np.exp(1j * int(round(k)) * basis.coordinates()))
    raise ValueError(f"{type(basis).__name__}: port {kind} is not available")


# --------------------------------------------------------------------------------------------
# Spec expressions and the term expansion (src/spec.jl, src/terms.jl:119-168)

_FUNCS = {"sqrt": math.sqrt, "cos": math.cos, "sin": math.sin, "exp": math.exp, "pi": math.pi,
          "π": math.pi, "log": math.log, "abs": abs, "tan": math.tan}


def eval_expr(x, theta):
    """A spec coefficient (number or expression string) evaluated at the parameters `theta`."""
    if isinstance(x, (int, float)) and not isinstance(x, bool):
        return float(x)
    src = str(x).replace("^", "**").replace("π", "pi")
    tree = ast.parse(src, mode="eval")

    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant):
            return float(node.value)
        if isinstance(node, ast.Name):
            if node.id in theta:
                return float(theta[node.id])
            if node.id in _FUNCS:
                return _FUNCS[node.id]
            raise KeyError(f"parameter {node.id} missing from theta")
        if isinstance(node, ast.BinOp):
            a, b = ev(node.left), ev(node.right)
            ops = {ast.Add: lambda: a + b, ast.Sub: lambda: a - b, ast.Mult: lambda: a * b,
                   ast.Div: lambda: a / b, ast.Pow: lambda: a ** b}
            if type(node.op) not in ops:
                raise ValueError(f"unsupported operator in {src}")
            return ops[type(node.op)]()
        if isinstance(node, ast.UnaryOp):
            v = ev(node.operand)
            return -v if isinstance(node.op, ast.USub) else v
        if isinstance(node, ast.Call):
            return ev(node.func)(*[ev(a) for a in node.args])
        raise ValueError(f"unsupported expression {src}")

    return ev(tree)


def load_spec(path_or_dict):
    if isinstance(path_or_dict, dict):
        return path_or_dict
    with open(path_or_dict) as f:
        return json.load(f)


def circuit_terms(spec, theta):
    """Expand a spec into numeric product terms (src/terms.jl:119-157).

    Returns a list of (coefficient: complex, [(mode_name, kind, k), ...]).  Terms whose
    coefficient is exactly zero are dropped.
    """
    names = [m["name"] for m in spec["modes"]]
    N = len(names)
    EC = [[eval_expr(spec["E_C"][i][j], theta) for j in range(N)] for i in range(N)]
    EL = [[eval_expr(spec["E_L"][i][j], theta) for j in range(N)] for i in range(N)]
    fl = [eval_expr(v, theta) for v in spec["flux_linear"]]
    ng = [eval_expr(v, theta) for v in spec["n_g"]]
    terms = []

    def add(c, fs):
        if c != 0:
            terms.append((complex(c), fs))

    for i in range(N):
        add(4 * EC[i][i], [(names[i], "n2", 0.0)])
    for i in range(N):
        for j in range(i + 1, N):
            add(4 * (EC[i][j] + EC[j][i]), [(names[i], "n", 0.0), (names[j], "n", 0.0)])
    for i in range(N):
        lin = sum((EC[i][j] + EC[j][i]) * ng[j] for j in range(N))
        add(-4 * lin, [(names[i], "n", 0.0)])
    for i in range(N):
        add(0.5 * EL[i][i], [(names[i], "phi2", 0.0)])
    for i in range(N):
        for j in range(i + 1, N):
            add(0.5 * (EL[i][j] + EL[j][i]), [(names[i], "phi", 0.0), (names[j], "phi", 0.0)])
    for i in range(N):
        add(fl[i], [(names[i], "phi", 0.0)])
    for c in spec.get("cosines", []):
        E = eval_expr(c["energy"], theta)
        off = eval_expr(c["offset"], theta)
        for s in (1, -1):
            fs = [(names[j], "expiphi", float(s * c["omega"][j])) for j in range(N) if c["omega"][j] != 0]
            add(-0.5 * E * np.exp(1j * s * off), fs)
    for c in spec.get("charge_cosines", []):
        E = eval_expr(c["energy"], theta)
        shift = sum(c["kappa"][j] * ng[j] for j in range(N))
        off = eval_expr(c["offset"], theta) - 2 * np.pi * shift
        for s in (1, -1):
            fs = [(names[j], "exp2pin", float(s * c["kappa"][j])) for j in range(N) if c["kappa"][j] != 0]
            add(-0.5 * E * np.exp(1j * s * off), fs)
    return terms


def constant_term(spec, theta):
    """constant + 4 n_g^T E_C n_g (src/terms.jl:164-168)."""
    names = spec["modes"]
    N = len(names)
    EC = [[eval_expr(spec["E_C"][i][j], theta) for j in range(N)] for i in range(N)]
    ng = [eval_expr(v, theta) for v in spec["n_g"]]
    const = eval_expr(spec.get("constant", 0), theta)
    return const + 4 * sum(ng[i] * EC[i][j] * ng[j] for i in range(N) for j in range(N))


# --------------------------------------------------------------------------------------------
# The real expansion of a product term (src/character.jl:281-315)

def _op_character(op):
    re, im = op.realpart(), op.imagpart()
    zr, zi = is_zero_op(re), is_zero_op(im)
    if zi:
        return "real", re, None
    if zr:
        return "imaginary", None, im
    return "paired", re, im


def _re_ipow(c, m):
    r = m % 4
    return float(c.real if r == 0 else -c.imag if r == 1 else -c.real if r == 2 else c.imag)


def real_expansion(coeff, factors):
    """Re(c ⊗_a O_a) as real terms Re(c i^|S|) ⊗_{a in S} I_a ⊗_{a not in S} R_a.

    `factors` is [(axis, op)]; returns [(coeff: float, [(axis, op)])], zero coefficients dropped.
    """
    comps = []
    for a, op in factors:
        kind, R, I = _op_character(op)
        choices = (False,) if kind == "real" else (True,) if kind == "imaginary" else (False, True)
        comps.append((a, R, I, choices))
    out = []

    def rec(idx, S):
        if idx == len(comps):
            c = _re_ipow(complex(coeff), sum(S))
            if c != 0:
                out.append((c, [(x[0], x[2] if s else x[1]) for x, s in zip(comps, S)]))
            return
        for ch in comps[idx][3]:
            rec(idx + 1, S + [ch])

    rec(0, [])
    return out


# --------------------------------------------------------------------------------------------
# apply_axis! (src/apply.jl:31-128)

def _axis_view(X, dims, k):
    """View of the flat column-major block X (N*b) as (left, d_k, right)."""
    left = int(np.prod(dims[:k])) if k > 0 else 1
    d = dims[k]
    return X.reshape((left, d, -1), order="F"), left, d


def apply_axis(op, X, dims, k):
    """Y = op applied along axis k (0-based) of the state block X (flat, column-major)."""
    Xr, left, d = _axis_view(X, dims, k)
    dt = np.result_type(X.dtype, _op_dtype(op))
    Y = np.zeros(Xr.shape, dtype=dt, order="F")
    if isinstance(op, DenseOp):
        Y[...] = np.einsum("ij,ljr->lir", op.M, Xr, optimize=True)
    elif isinstance(op, DiagonalOp):
        Y[...] = op.d[None, :, None] * Xr
    elif isinstance(op, BandedOp):
        for o, w in zip(op.offsets, op.weights):
            lo, hi = max(0, -o), min(d, d - o)          # rows i with 0 <= i + o < d
            if lo < hi:
                Y[:, lo:hi, :] += w[lo:hi][None, :, None] * Xr[:, lo + o:hi + o, :]
    elif isinstance(op, ShiftOp):
        s = op.s
        lo, hi = max(0, s), min(d, d + s)               # rows i with 0 <= i - s < d
        if lo < hi:
            Y[:, lo:hi, :] = op.factor * Xr[:, lo - s:hi - s, :]
    else:
        raise TypeError(type(op))
    return Y.reshape(-1, order="F")


def _op_dtype(op):
    if isinstance(op, DenseOp):
        return op.M.dtype
    if isinstance(op, DiagonalOp):
        return op.d.dtype
    if isinstance(op, BandedOp):
        return op.weights[0].dtype if op.weights else np.float64
    return np.result_type(op.factor, np.float64)


# --------------------------------------------------------------------------------------------
# KronFreeOperator (src/apply.jl:175-685)

class KronFreeOperator:
    """H = sum_t c_t ⊗_k A_{t,k} + constant I, axis 1 fastest (src/apply.jl:222-253).

    `terms` is a list of (coeff, [(axis, op), ...]) with 0-based, strictly increasing axes.
    All-diagonal terms and the constant are fused into `self.diag`; the rest are kept.
    """

    def __init__(self, dims, terms, constant=0.0):
        self.dims = [int(d) for d in dims]
        if any(d < 1 for d in self.dims):
            raise ValueError("dims must be positive")
        cplx = np.iscomplexobj(constant) and complex(constant).imag != 0
        for c, fs in terms:
            axes = [a for a, _ in fs]
            if any(b <= a for a, b in zip(axes, axes[1:])):
                raise ValueError("factor axes must be strictly increasing")
            for a, op in fs:
                if not 0 <= a < len(self.dims):
                    raise ValueError(f"factor axis {a} out of range")
                if op.n != self.dims[a]:
                    raise ValueError(f"factor on axis {a} has dimension {op.n}, expected {self.dims[a]}")
            cplx = cplx or (np.iscomplexobj(c) and complex(c).imag != 0) or \
                any(np.dtype(_op_dtype(op)).kind == "c" for _, op in fs)
        self.dtype = np.complex128 if cplx else np.float64
        self.N = int(np.prod(self.dims))
        constant = _scalar(constant, self.dtype)
        D = np.full(self.dims, constant, dtype=self.dtype, order="F")
        self.diagterms = [(constant, [])] if constant != 0 else []
        self.terms = []
        for c, fs in terms:
            if all(isinstance(op, DiagonalOp) for _, op in fs):
                D += _kron_diag(self.dims, c, fs, self.dtype)
                self.diagterms.append((c, fs))
            else:
                self.terms.append((_scalar(c, self.dtype), fs))
        self.diag = D.reshape(-1, order="F")

    @property
    def shape(self):
        return (self.N, self.N)

    def matvec(self, x):
        """mul!(y, H, x) (src/apply.jl:416-432): fused diagonal, then one chained pass per term."""
        x = np.asarray(x)
        vec = x.ndim == 1
        X = x.reshape(self.N, -1, order="F")
        b = X.shape[1]
        dims = self.dims + [b]
        flat = X.reshape(-1, order="F")
        dt = np.result_type(self.dtype, x.dtype)
        Y = (np.tile(self.diag, b) * flat).astype(dt)
        for c, fs in self.terms:
            src = flat
            for a, op in fs:
                src = apply_axis(op, src, dims, a)
            Y += c * src
        Y = Y.reshape(self.N, b, order="F")
        return Y[:, 0] if vec else Y

    __matmul__ = matvec

    def to_matrix(self):
        """Matrix(H): H applied to identity blocks of at most 256 columns (src/apply.jl:506-531)."""
        n = self.N
        M = np.empty((n, n), dtype=self.dtype)
        for c0 in range(0, n, 256):
            w = min(256, n - c0)
            E = np.zeros((n, w), dtype=self.dtype)
            E[c0 + np.arange(w), np.arange(w)] = 1
            M[:, c0:c0 + w] = self.matvec(E)
        return M

    def diagonal(self):
        """The full diagonal (src/apply.jl:455-470)."""
        D = self.diag.reshape(self.dims, order="F").copy()
        for c, fs in self.terms:
            acc = np.full([1] * len(self.dims), c, dtype=self.dtype)
            for a, op in fs:
                shp = [1] * len(self.dims)
                shp[a] = self.dims[a]
                acc = acc * op.diagonal().reshape(shp)
            D = D + acc
        return D.reshape(-1, order="F")

    def full_diagonal(self):
        return np.real(self.diagonal())

    def gershgorin_bound(self):
        """max Re(diag) + max |Im diag| + sum_t |c_t| prod infnorm (src/apply.jl:586-593)."""
        off = sum(abs(c) * float(np.prod([op.infnorm() for _, op in fs])) for c, fs in self.terms)
        return float(np.max(np.real(self.diag)) + np.max(np.abs(np.imag(self.diag))) + off)

    def separable_eigenbases(self):
        """Per-axis eigenbases of the single-axis terms (src/apply.jl:606-642)."""
        A = [np.zeros((d, d), dtype=self.dtype) for d in self.dims]
        for c, fs in self.terms:
            if len(fs) == 1:
                a, op = fs[0]
                A[a] += c * op.dense()
        for c, fs in self.diagterms:
            if len(fs) == 1:
                a, op = fs[0]
                A[a] += c * op.dense()
            elif len(fs) == 0:
                A[0] += c * np.eye(self.dims[0])
        U, lam = [], []
        for M in A:
            if np.linalg.norm(M - M.conj().T) > math.sqrt(np.finfo(float).eps) * np.linalg.norm(M):
                raise ValueError("separable_eigenbases: non-Hermitian single-axis sum")
            if not np.any(M - np.diag(np.diag(M))):
                U.append(None)                       # identity
                lam.append(np.real(np.diag(M)).copy())
            else:
                w, V = np.linalg.eigh((M + M.conj().T) / 2)
                U.append(V)
                lam.append(w)
        return U, lam

    def product_seed(self, k):
        """k orthonormal product states of lowest separable energy (src/apply.jl:655-685).

        Ties are broken by the flat index (a stable sort), the order Julia's partialsortperm
        gives for the cases the goldens pin.
        """
        n = self.N
        if not 1 <= k <= n:
            raise ValueError(f"product_seed: k must lie in 1:{n}")
        U, lam = self.separable_eigenbases()
        X = np.zeros((n, k), dtype=self.dtype)
        if all(u is None for u in U):
            idx = np.argsort(self.full_diagonal(), kind="stable")[:k]
            X[idx, np.arange(k)] = 1
            return X
        sums = lam[0]
        for a in range(1, len(self.dims)):
            sums = (sums[:, None] + lam[a][None, :]).reshape(-1, order="F")
        order = np.argsort(sums, kind="stable")[:k]
        for j, flat in enumerate(order):
            idx = np.unravel_index(flat, self.dims, order="F")
            v = np.ones(1, dtype=self.dtype)
            for a in range(len(self.dims)):
                ua = np.eye(self.dims[a])[:, idx[a]] if U[a] is None else U[a][:, idx[a]]
                v = np.kron(ua, v)
            X[:, j] = v
        return X


def _scalar(c, dtype):
    c = complex(c)
    return c.real if dtype is np.float64 else c


def _kron_diag(dims, c, fs, dtype):
    acc = np.full([1] * len(dims), _scalar(c, dtype), dtype=dtype)
    for a, op in fs:
        shp = [1] * len(dims)
        shp[a] = dims[a]
        acc = acc * op.d.reshape(shp)
    return np.broadcast_to(acc, dims)


def kron_reference(dims, terms, constant=0.0):
    """Dense sum_t c_t A_{t,N} ⊗ ... ⊗ A_{t,1} (test/helpers.jl:10-24), axis 1 fastest."""
    n = int(np.prod(dims))
    H = constant * np.eye(n, dtype=np.complex128)
    for c, fs in terms:
        ops = {a: op.dense() for a, op in fs}
        T = np.ones((1, 1), dtype=np.complex128)
        for a, d in enumerate(dims):
            T = np.kron(ops.get(a, np.eye(d)), T)
        H = H + c * T
    return H


# --------------------------------------------------------------------------------------------
# A leaf node's operator from a spec (the leaf case of src/materialize.jl:583-647)

def leaf_terms(spec, theta, bases, modes=None, real=False):
    """The product terms of `spec` on a flat product of `bases` (mode name -> basis, axis order).

    Every term whose modes all lie among `bases` is kept (a leaf takes every term routed to it;
    with `modes` given, only terms whose modes are all in `modes`).  With `real=True` each term is
    replaced by its real expansion (src/character.jl:297-315) and equal real terms are summed.
    """
    names = list(bases.keys())
    allowed = set(modes) if modes is not None else set(names)
    out = []
    for c, fs in circuit_terms(spec, theta):
        if not all(m in allowed for m, _, _ in fs):
            continue
        factors = sorted([(names.index(m), localop(bases[m], kind, k)) for m, kind, k in fs], key=lambda t: t[0])
        if real:
            out.extend(real_expansion(c, factors))
        else:
            out.append((c, factors))
    return out
