"""kfgpu: the GB300 Kronecker-free operator and eigensolvers of KronFreeCircuits.jl.

The compute path is libkfgpu.so (hand-written sm_103a CUDA behind a C ABI, include/kfgpu.h);
this package is its host-side mirror of the reference's interface: local operators and bases
(`ops`), `KronFreeOperator` (`operator`), the solver option structs and `solve` (`solvers`).
The library must be built (`kfgpu.build.build_library()`); without it every call raises.
"""
from ._abi import (ArgumentError, ConvergenceError, DimensionMismatch, KFError, lib)
from .operator import KronFreeOperator
from .ops import BandedOp, ChargeBasis, DenseOp, DiagonalOp, PhaseGrid, ShiftOp, localop
from .solvers import ChebyshevFilter, Lanczos, LOBPCG, solve

__all__ = ["ArgumentError", "ConvergenceError", "DimensionMismatch", "KFError", "lib", "KronFreeOperator",
           "BandedOp", "ChargeBasis", "DenseOp", "DiagonalOp", "PhaseGrid", "ShiftOp", "localop",
           "ChebyshevFilter", "Lanczos", "LOBPCG", "solve"]
