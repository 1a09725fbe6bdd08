"""The reference's solver option structs and `solve`, over libkfgpu's kf_solve.

  LOBPCG(; tol, maxiter, preconditioner, eta, guard, seed)             src/tree.jl:66-87
  ChebyshevFilter(; tol, degree, extra, maxiter, rescale_every, ortho, bound, seed)   src/tree.jl:293-321
  Lanczos(; tol, krylovdim, maxiter)                                    src/tree.jl:15-23
  solve(s, H, m; X0) -> (E, V)                                          src/solvers.jl:6-31

Each option struct also takes `precision` ("f64": every step in FP64; "mixed": FP32 bulk with
FP64 Rayleigh-Ritz and FP64 refinement), validated like the reference's constructors.
`solve` returns host arrays and a stats dict (iterations, n_matvec, residual, timings).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from ._abi import ArgumentError, check, lib

_PREC = {"f64": _abi.KF_PREC_F64, "mixed": _abi.KF_PREC_MIXED}


def _arg(cond, msg):
    if not cond:
        raise ArgumentError(_abi.KF_EINVAL, msg)


class LOBPCG:
    def __init__(self, tol=1e-8, maxiter=1000, preconditioner="ritz", eta=0.01, guard=4, seed="product",
                 precision="f64", mixed_switch=1e-6, fallback_iters=3, fallback_resid=0.0, rng_seed=0x4B46,
                 buffer=None):
        _arg(tol > 0 and math.isfinite(tol), f"LOBPCG: tol must be positive and finite, got {tol}")
        _arg(maxiter >= 1, f"LOBPCG: maxiter must be at least 1, got {maxiter}")
        _arg(preconditioner in ("ritz", "jacobi", "none", "separable"),
             f"LOBPCG: preconditioner must be :ritz, :jacobi, :none or :separable, got :{preconditioner}")
        _arg(eta > 0 and math.isfinite(eta), f"LOBPCG: eta must be positive and finite, got {eta}")
        _arg(guard >= 0, f"LOBPCG: guard must be nonnegative, got {guard}")
        _arg(seed in ("product", "random"), f"LOBPCG: seed must be :product or :random, got {seed!r}")
        _arg(precision in _PREC, f"LOBPCG: precision must be f64 or mixed, got {precision!r}")
        _arg(buffer is None or buffer >= 0, f"LOBPCG: buffer must be nonnegative, got {buffer}")
        self.tol, self.maxiter, self.preconditioner, self.eta = tol, maxiter, preconditioner, eta
        self.guard, self.seed, self.precision = guard, seed, precision
        self.mixed_switch, self.fallback_iters, self.fallback_resid = mixed_switch, fallback_iters, fallback_resid
        self.rng_seed = rng_seed
        # unchecked columns beyond the guards (None: the library's choice, 2 for mixed, 0 for f64)
        self.buffer = buffer

    def opts(self):
        o = _abi.KfSolverOpts()
        lib().kf_solver_opts_default(C.byref(o), _abi.KF_SOLVER_LOBPCG)
        o.buffer = _abi.KF_BUFFER_AUTO if self.buffer is None else self.buffer
        o.precision, o.tol, o.maxiter = _PREC[self.precision], self.tol, self.maxiter
        o.preconditioner = {"ritz": 0, "jacobi": 1, "none": 2, "separable": 3}[self.preconditioner]
        o.eta, o.guard, o.mixed_switch = self.eta, self.guard, self.mixed_switch
        o.fallback_iters, o.fallback_resid, o.rng_seed = self.fallback_iters, self.fallback_resid, self.rng_seed
        o.seed_kind = _abi.KF_SEED_PRODUCT if self.seed == "product" else _abi.KF_SEED_RANDOM
        return o

    def width(self, N, m):
        return m + min(self.guard, (N - 5) // 3 - m)


class ChebyshevFilter:
    def __init__(self, tol=1e-8, degree=100, extra=40, maxiter=50, rescale_every=20, ortho="svqb",
                 bound="gershgorin", seed="product", precision="f64", rng_seed=0x4346):
        _arg(tol > 0 and math.isfinite(tol), f"ChebyshevFilter: tol must be positive and finite, got {tol}")
        _arg(1 <= degree <= 200, f"ChebyshevFilter: degree must lie in 1:200, got {degree}")
        _arg(extra >= 2, "ChebyshevFilter: extra must be at least 2 so at least one column serves as a convergence "
                         f"guard; the top column sets the filter cut and cannot be one, got {extra}")
        _arg(maxiter >= 1, f"ChebyshevFilter: maxiter must be at least 1, got {maxiter}")
        _arg(rescale_every >= 1, f"ChebyshevFilter: rescale_every must be at least 1, got {rescale_every}")
        _arg(ortho in ("svqb", "cholqr"), f"ChebyshevFilter: ortho must be :svqb or :cholqr, got {ortho!r}")
        _arg(bound == "gershgorin" or (isinstance(bound, (int, float)) and math.isfinite(bound)),
             f"ChebyshevFilter: bound must be :gershgorin or a finite number, got {bound!r}")
        _arg(seed in ("product", "random"), f"ChebyshevFilter: seed must be :product or :random, got {seed!r}")
        _arg(precision in _PREC, f"ChebyshevFilter: precision must be f64 or mixed, got {precision!r}")
        self.tol, self.degree, self.extra, self.maxiter = tol, degree, extra, maxiter
        self.rescale_every, self.ortho, self.bound, self.seed = rescale_every, ortho, bound, seed
        self.precision, self.rng_seed = precision, rng_seed

    def opts(self):
        o = _abi.KfSolverOpts()
        lib().kf_solver_opts_default(C.byref(o), _abi.KF_SOLVER_CHEBYSHEV)
        o.precision, o.tol, o.maxiter = _PREC[self.precision], self.tol, self.maxiter
        o.degree, o.extra, o.rescale_every = self.degree, self.extra, self.rescale_every
        o.ortho = 0 if self.ortho == "svqb" else 1
        o.bound = float("nan") if self.bound == "gershgorin" else float(self.bound)
        o.seed_kind = _abi.KF_SEED_PRODUCT if self.seed == "product" else _abi.KF_SEED_RANDOM
        o.rng_seed = self.rng_seed
        return o

    def width(self, N, m):
        return min(m + self.extra, N)


class Lanczos:
    def __init__(self, tol=1e-10, krylovdim=0, maxiter=1000, rng_seed=0x4C41):
        _arg(tol > 0 and math.isfinite(tol), f"Lanczos: tol must be positive and finite, got {tol}")
        _arg(krylovdim >= 0 and maxiter >= 1, "Lanczos: krylovdim must be nonnegative and maxiter at least 1")
        self.tol, self.krylovdim, self.maxiter, self.rng_seed = tol, krylovdim, maxiter, rng_seed
        self.seed = "random"

    def opts(self):
        o = _abi.KfSolverOpts()
        lib().kf_solver_opts_default(C.byref(o), _abi.KF_SOLVER_LANCZOS)
        o.tol, o.maxiter, o.krylovdim, o.rng_seed = self.tol, self.maxiter, self.krylovdim, self.rng_seed
        return o


def solve(s, H, m, X0=None, seed_block=None):
    """The lowest m eigenpairs of H: (E ascending, V N x m host, stats dict).

    With `s.seed == "product"` the library builds product_seed(H, w) on the device, as the
    reference's solve does (src/lobpcg.jl:247); `seed_block` (N x w, host) replaces it.
    """
    N = H.N
    o = s.opts()
    seed_arr = None
    if not isinstance(s, Lanczos) and seed_block is not None:
        seed_arr = np.asfortranarray(seed_block, dtype=np.float64)
    x0 = None
    if X0 is not None:
        x0 = np.asfortranarray(X0, dtype=np.float64)
        if x0.shape != (N, m):
            raise _abi.DimensionMismatch(_abi.KF_EDIM, f"LOBPCG: X0 has size {x0.shape}, expected ({N}, {m})")
    E = np.empty(max(m, 1))
    V = np.empty((N, max(m, 1)), order="F")
    st = _abi.KfSolveStats()
    status = lib().kf_solve(H.handle, C.byref(o), int(m), x0.ctypes.data if x0 is not None else None,
                            seed_arr.ctypes.data if seed_arr is not None else None, E.ctypes.data, V.ctypes.data,
                            C.byref(st))
    stats = st.as_dict()
    if status != _abi.KF_OK:
        try:
            check(status)
        except _abi.KFError as e:
            e.stats = stats
            raise
    return E[:m], V[:, :m], stats
