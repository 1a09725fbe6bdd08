"""Ports as operators on a node's product basis.

  port_operator(sys, key, node)        src/portoperator.jl:18-39
  port_matrix(H, V, W)                 src/materialize.jl:426-517 (_apply_ops, _port_matrix,
                                       _node_port, _joint_port, _real_sandwich): W' H V on the GPU

The reference's `port_operator` returns a one-term `KronFreeOperator` (coefficient 1, one factor
per keyed mode, identity on the other axes) on the product basis of `node`; each factor is the
child's stored port (a dense matrix in the child's kept basis) or, for a leaf mode, the basis
operator.  Here the caller (the Julia shim, which owns the tree) passes the node's axis dimensions
and the factors as (axis, op) pairs; the operator lives on the GPU like any `kf_op`, so its
application is the same fused / chained `mul!`.  Real factors only (diagonal, banded, shift and
dense real matrices): every configuration measured here is real by structure.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .operator import KronFreeOperator


def _hermitian(op):
    """Whether a factor is Hermitian to rounding (src/portoperator.jl:37: isapprox(M, M'; rtol 1e-10,
    atol 1e-12 max(1, ||M||_inf)))."""
    M = op.dense()
    scale = max(1.0, float(np.max(np.sum(np.abs(M), axis=1))) if M.size else 1.0)
    return bool(np.all(np.abs(M - M.T) <= 1e-10 * np.abs(M) + 1e-12 * scale))


def port_operator(dims, key, block_capacity=1):
    """The port `key` = [(axis, op)] (one factor, or a joint port of factors on distinct axes) as a
    one-term operator on the product basis with axis dimensions `dims`; `.hermitian` tells whether
    every factor is Hermitian (so the operator is)."""
    key = list(key)
    if not key:
        raise _abi.ArgumentError(_abi.KF_EINVAL, "port_operator: the key is empty")
    for a, op in key:
        if not 0 <= a < len(dims):
            raise _abi.ArgumentError(_abi.KF_EINVAL, f"mode {a} is not a mode of the node with axes 0:{len(dims) - 1}")
    key.sort(key=lambda t: t[0])
    axes = [a for a, _ in key]
    if len(set(axes)) != len(axes):
        raise _abi.ArgumentError(
            _abi.KF_EINVAL, f"port_operator: the factors of a joint key must be on distinct modes, got axes {axes}")
    H = KronFreeOperator(dims, [(1.0, key)], block_capacity=block_capacity)
    H.hermitian = all(_hermitian(op) for _, op in key)
    return H


def port_matrix(H, V, W=None):
    """W' H V (host FP64, kw x kv) for host blocks V (N x kv) and W (N x kw, default V): a port or
    joint port of a node's kept vectors V when H is its port operator, one component of a real
    expansion when H carries that component's terms (kf_op_sandwich)."""
    Vf = np.asfortranarray(V, dtype=np.float64)
    if Vf.ndim != 2 or Vf.shape[0] != H.N:
        raise _abi.DimensionMismatch(_abi.KF_EDIM, f"port_matrix: V has shape {Vf.shape}, expected ({H.N}, k)")
    Wf = None if W is None else np.asfortranarray(W, dtype=np.float64)
    if Wf is not None and (Wf.ndim != 2 or Wf.shape[0] != H.N):
        raise _abi.DimensionMismatch(_abi.KF_EDIM, f"port_matrix: W has shape {Wf.shape}, expected ({H.N}, k)")
    kw = Vf.shape[1] if Wf is None else Wf.shape[1]
    P = np.empty((kw, Vf.shape[1]), order="F")
    _abi.check(_abi.lib().kf_op_sandwich(H.handle, None if Wf is None else Wf.ctypes.data, H.N, kw, Vf.ctypes.data,
                                         H.N, Vf.shape[1], P.ctypes.data, _abi.KF_HOST))
    return P
