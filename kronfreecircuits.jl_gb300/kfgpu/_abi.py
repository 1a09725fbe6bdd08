"""ctypes binding of libkfgpu.so (the C ABI in include/kfgpu.h).

The library is loaded from this package directory only (it is built in-tree by
`kfgpu.build.build_library`).  A missing or unloadable library raises ImportError at first
use: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# KF_LIB selects another build of the library (the bounds-recording libkfgpu_check.so)
LIB_PATH = os.environ.get("KF_LIB") or os.path.join(_HERE, "libkfgpu.so")

KF_OK, KF_EINVAL, KF_EDIM, KF_EALIAS, KF_ECUDA, KF_ENOCONV, KF_EBREAKDOWN, KF_ENOMEM, KF_ETIMEOUT, KF_ENOTFINITE = range(10)
KF_F64, KF_F32, KF_HOST = 0x0, 0x1, 0x2
KF_DEVICE = 0x0
KF_DIAG, KF_BANDED, KF_SHIFT, KF_DENSE = range(4)
KF_SOLVER_LOBPCG, KF_SOLVER_CHEBYSHEV, KF_SOLVER_LANCZOS = range(3)
KF_PREC_F64, KF_PREC_MIXED = 0, 1
KF_PRECOND_RITZ, KF_PRECOND_JACOBI, KF_PRECOND_NONE, KF_PRECOND_SEPARABLE = range(4)
KF_ORTHO_SVQB, KF_ORTHO_CHOLQR = 0, 1


class KfFactor(C.Structure):
    _fields_ = [("axis", C.c_int32), ("kind", C.c_int32), ("n", C.c_int64), ("data", C.POINTER(C.c_double)),
                ("offsets", C.POINTER(C.c_int64)), ("nbands", C.c_int32), ("shift", C.c_int64),
                ("factor", C.c_double)]


class KfTerm(C.Structure):
    _fields_ = [("coeff", C.c_double), ("nfactors", C.c_int32), ("factors", C.POINTER(KfFactor))]


class KfOpDesc(C.Structure):
    _fields_ = [("ndims", C.c_int32), ("dims", C.POINTER(C.c_int64)), ("constant", C.c_double),
                ("nterms", C.c_int32), ("terms", C.POINTER(KfTerm)), ("diag", C.POINTER(C.c_double)),
                ("block_capacity", C.c_int64)]


KF_SEED_PRODUCT, KF_SEED_RANDOM = 0, 1
KF_BUFFER_AUTO = -1


class KfSolverOpts(C.Structure):
    _fields_ = [("kind", C.c_int32), ("precision", C.c_int32), ("tol", C.c_double), ("maxiter", C.c_int32),
                ("preconditioner", C.c_int32), ("eta", C.c_double), ("guard", C.c_int32), ("degree", C.c_int32),
                ("extra", C.c_int32), ("rescale_every", C.c_int32), ("ortho", C.c_int32), ("bound", C.c_double),
                ("krylovdim", C.c_int32), ("rng_seed", C.c_uint64), ("mixed_switch", C.c_double),
                ("fallback_iters", C.c_int32), ("fallback_resid", C.c_double), ("seed_kind", C.c_int32),
                ("buffer", C.c_int32)]


class KfSolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("iterations_f64", C.c_int32), ("n_matvec", C.c_int64),
                ("warm", C.c_int32), ("fell_back", C.c_int32), ("converged", C.c_int32),
                ("max_residual", C.c_double), ("hnorm", C.c_double), ("seconds", C.c_double),
                ("seconds_f64", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class KFError(RuntimeError):
    """A failed libkfgpu call; `code` is the KF_E* status."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class ArgumentError(KFError, ValueError):
    """The reference's ArgumentError."""


class DimensionMismatch(KFError, ValueError):
    """The reference's DimensionMismatch."""


class ConvergenceError(KFError):
    """An eigensolver did not converge (the reference's ErrorException)."""


_lib = None


def lib():
    """The loaded libkfgpu.so (ImportError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libkfgpu.so is not built ({LIB_PATH}); run kfgpu.build.build_library()")
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    sig = {
        "kf_version": (C.c_int, []),
        "kf_launch_count": (C.c_int, [C.POINTER(C.c_uint64)]),
        "kf_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
        "kf_op_create": (C.c_int, [C.POINTER(KfOpDesc), C.POINTER(P)]),
        "kf_op_destroy": (C.c_int, [P]),
        "kf_op_size": (C.c_int, [P, C.POINTER(C.c_int64)]),
        "kf_op_apply": (C.c_int, [P, P, P, C.c_int64, C.c_int64, C.c_int64, C.c_int32]),
        "kf_op_apply_noalloc": (C.c_int, [P, P, P, C.c_int64, C.c_int64, C.c_int64, C.c_int32]),
        "kf_op_apply_axpby": (C.c_int, [P, P, P, P, C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double,
                                        C.c_int32]),
        "kf_op_sandwich": (C.c_int, [P, P, C.c_int64, C.c_int32, P, C.c_int64, C.c_int32, P, C.c_int32]),
        "kf_complement_solve": (C.c_int, [P, P, C.c_int64, C.c_int32, P, C.c_int64, C.c_int32, P, P, C.c_double,
                                          C.c_int32, C.c_double, P, C.c_int64, P, P, P, P, C.c_int32]),
        "kf_drive_apply": (C.c_int, [P, C.c_double, C.c_int32, P, P, P, P, C.c_double, P, C.c_int64, P, C.c_int64,
                                     C.c_int64, C.c_int32]),
        "kf_to_lab": (C.c_int, [P, C.c_int64, C.c_double, P, C.c_int64, C.c_int64, C.c_int32]),
        "kf_op_diagonal": (C.c_int, [P, C.POINTER(C.c_double)]),
        "kf_op_gershgorin": (C.c_int, [P, C.POINTER(C.c_double)]),
        "kf_op_get_stream": (C.c_int, [P, C.POINTER(P)]),
        "kf_op_set_stream": (C.c_int, [P, P]),
        "kf_op_sync": (C.c_int, [P]),
        "kf_op_product_seed": (C.c_int, [P, C.c_int32, P, C.c_int32]),
        "kf_solver_opts_default": (None, [C.POINTER(KfSolverOpts), C.c_int32]),
        "kf_solve": (C.c_int, [P, C.POINTER(KfSolverOpts), C.c_int32, P, P, P, P, C.POINTER(KfSolveStats)]),
        "kf_batch_solve": (C.c_int, [C.POINTER(KfOpDesc), C.c_int32, C.POINTER(C.c_int32), C.c_double, C.c_int32,
                                     C.c_int32, P, P, P, P]),
        "kf_batch_autotune": (C.c_int, [C.POINTER(KfOpDesc), C.c_int32, C.POINTER(C.c_int32), C.c_double,
                                        C.c_int32, C.POINTER(C.c_int32)]),
        "kf_mlp_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(P)]),
        "kf_mlp_destroy": (C.c_int, [P]),
        "kf_mlp_set_scaling": (C.c_int, [P, P, P, P, P]),
        "kf_mlp_train": (C.c_int, [P, P, P, C.c_int64, C.c_int32, C.c_int32, C.c_float, C.c_uint64, P]),
        "kf_mlp_forward": (C.c_int, [P, P, P, C.c_int64]),
        "kf_mlp_gradients": (C.c_int, [P, P, P, C.c_int64, P, P]),
        "kf_mlp_get_params": (C.c_int, [P, P, C.POINTER(C.c_int64)]),
        # test-only (include/kfgpu_testing.h)
        "kf_test_mode_product": (C.c_int, [C.c_int32, P, P, P, C.c_int32, C.c_int64, C.c_int64, C.c_int64,
                                           C.c_double, C.c_double, P]),
        "kf_test_time_mode_product": (C.c_int, [C.c_int32, P, P, P, C.c_int32, C.c_int64, C.c_int64, C.c_int64,
                                                C.c_int32, P, C.POINTER(C.c_float)]),
        "kf_test_time_gram": (C.c_int, [C.c_int32, P, C.c_int64, C.c_int32, P, C.c_int64, C.c_int32, C.c_int64, C.c_int32, P,
                                        C.POINTER(C.c_float), P]),
        "kf_test_chol2": (C.c_int, [P, C.c_int32, C.c_int32, P, P]),
        "kf_test_op_scratch_bytes": (C.c_int, [P, P]),
        "kf_test_check_word": (C.c_int, [P, P]),
        "kf_test_rr_eig": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P]),
        "kf_test_march_plan": (C.c_int, [P, C.c_int64, C.c_int32, C.c_int32, P, P]),
        "kf_test_sym_eig": (C.c_int, [C.c_int32, P, C.c_int32, P, P, C.c_int32]),
        "kf_test_update_split": (C.c_int, [C.c_int32, P, C.c_int32, P, C.c_int32, P, C.c_int32, P, C.c_int32, P, C.c_double,
                                           C.c_double, C.c_int64, C.c_int64]),
        "kf_test_update_f64": (C.c_int, [C.c_int32, P, P, C.c_int32, C.c_int32, P, C.c_int64, C.c_int32, P,
                                         C.POINTER(C.c_float)]),
        "kf_test_gram_tc": (C.c_int, [P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64,
                                      C.c_int32, P, C.POINTER(C.c_float), P]),
        "kf_test_apply_variant": (C.c_int, [P, C.c_int32, P, P, C.c_int64, C.c_int64, C.c_int32, C.c_int32,
                                            C.POINTER(C.c_float)]),
        "kf_test_update": (C.c_int, [C.c_int32, P, C.c_int64, C.c_int32, P, C.c_int64, C.c_int32, P, C.c_int64,
                                     C.c_int32, P, C.c_int32, C.c_double, C.c_double, C.c_int64, C.c_int32, P,
                                     C.POINTER(C.c_float)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def launch_count():
    """Kernels libkfgpu has launched in this process."""
    v = C.c_uint64()
    lib().kf_launch_count(C.byref(v))
    return v.value


def last_error():
    buf = C.create_string_buffer(4096)
    lib().kf_last_error(buf, 4096)
    return buf.value.decode("utf-8", "replace")


def check(status):
    """Raise the exception matching a non-zero status, with the library's message."""
    if status == KF_OK:
        return
    msg = last_error()
    if status == KF_EINVAL or status == KF_EALIAS:
        raise ArgumentError(status, msg)
    if status == KF_EDIM:
        raise DimensionMismatch(status, msg)
    if status in (KF_ENOCONV, KF_EBREAKDOWN, KF_ENOTFINITE, KF_ETIMEOUT):
        raise ConvergenceError(status, msg)
    raise KFError(status, msg)
