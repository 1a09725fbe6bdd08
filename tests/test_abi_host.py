"""CPU tests of the C ABI and the host-side mirror: the library loads and exports every symbol
include/kfgpu.h declares, option structs validate like the reference's constructors, and the
host-built term lists equal the oracle's spec-built Hamiltonians (no GPU calls)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from oracle import circuits as ocirc
from oracle import kfref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    syms = set()
    for h in sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))):
        with open(h) as f:
            src = f.read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        syms |= set(re.findall(r"\b(kf_[a-z0-9_]+)\s*\(", src))
    return sorted(syms)


def test_library_builds_and_exports_every_declared_symbol():
    from kfgpu.build import build_library
    path = build_library()
    lib = ctypes.CDLL(path)
    syms = _declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.kf_version() == 1


def test_python_binding_covers_every_symbol():
    from kfgpu import _abi
    L = _abi.lib()
    for s in _declared_symbols():
        assert getattr(L, s).argtypes is not None or s == "kf_version", s


def test_struct_layouts_match_header():
    """Sizes of the ctypes mirrors equal the C structs (compiled probe of the header)."""
    import subprocess, tempfile
    from kfgpu import _abi
    src = '#include "kfgpu.h"\n#include <stdio.h>\nint main(){printf("%zu %zu %zu %zu %zu\\n", sizeof(kf_factor),' \
          ' sizeof(kf_term), sizeof(kf_op_desc), sizeof(kf_solver_opts), sizeof(kf_solve_stats));}\n'
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        sizes = [int(x) for x in subprocess.check_output([exe]).split()]
    assert sizes == [ctypes.sizeof(_abi.KfFactor), ctypes.sizeof(_abi.KfTerm), ctypes.sizeof(_abi.KfOpDesc),
                     ctypes.sizeof(_abi.KfSolverOpts), ctypes.sizeof(_abi.KfSolveStats)]


def test_solver_option_validation():
    from kfgpu import ArgumentError, ChebyshevFilter, LOBPCG
    with pytest.raises(ArgumentError):
        LOBPCG(tol=0)
    with pytest.raises(ArgumentError):
        LOBPCG(preconditioner="magic")
    with pytest.raises(ArgumentError):
        LOBPCG(guard=-1)
    with pytest.raises(ArgumentError):
        LOBPCG(buffer=-1)
    # buffer columns: the library's choice unless given; never part of the returned width
    from kfgpu import _abi
    assert LOBPCG().opts().buffer == _abi.KF_BUFFER_AUTO
    assert LOBPCG(buffer=3).opts().buffer == 3
    assert LOBPCG(buffer=3).width(671744, 12) == 16
    with pytest.raises(ArgumentError):
        ChebyshevFilter(extra=1)
    with pytest.raises(ArgumentError):
        ChebyshevFilter(degree=201)
    with pytest.raises(ArgumentError):
        ChebyshevFilter(bound=float("inf"))
    assert LOBPCG().width(671744, 12) == 16
    assert LOBPCG().width(40, 10) == 10 + min(4, (40 - 5) // 3 - 10)


def _dense_from_terms(dims, terms, constant=0.0):
    n = int(np.prod(dims))
    H = constant * np.eye(n)
    for c, fs in terms:
        ops = {a: op.dense() for a, op in fs}
        T = np.ones((1, 1))
        for a, d in enumerate(dims):
            T = np.kron(ops.get(a, np.eye(d)), T)
        H = H + c * T
    return H


def test_three_mode_terms_match_oracle_spec():
    """The product's hand-written term list equals the spec route (circuit_terms + real expansion)."""
    from kfgpu import circuits
    th = ocirc.three_mode_theta(np.random.default_rng(7))
    dims, terms = circuits.three_mode_leaf(th, ncut=3, n2=12, n3=9)
    Ho = ocirc.three_mode_operator(th, ncut=3, n2=12, n3=9).to_matrix()
    assert np.allclose(_dense_from_terms(dims, terms), Ho, atol=1e-12)


def test_fluxonium_terms_match_oracle_spec():
    from kfgpu import circuits
    th = ocirc.fluxonium_theta(np.random.default_rng(8)) if hasattr(ocirc, "fluxonium_theta") else \
        {"E_J": 5.0, "E_C": 1.1, "E_L": 0.7, "phi_ext": 1.3}
    dims, terms = circuits.fluxonium_leaf(th, 40)
    Ho = ocirc.fluxonium_operator(th, 40).to_matrix()
    assert np.allclose(_dense_from_terms(dims, terms), Ho, atol=1e-12)


def test_two_transmon_flat_matches_oracle_spec(goldens):
    from kfgpu import circuits
    th = goldens["goldens"]["two_transmons"]["params"]
    dims, terms, const = circuits.two_transmon_flat(th, ncut=4)
    bases = {"varphi_1": kfref.ChargeBasis(4), "varphi_2": kfref.ChargeBasis(4)}
    spec = goldens["specs"]["two_transmons"]
    Ho = kfref.KronFreeOperator([9, 9], kfref.leaf_terms(spec, th, bases, real=True),
                                constant=kfref.constant_term(spec, th)).to_matrix()
    assert np.allclose(_dense_from_terms(dims, terms, const), Ho, atol=1e-12)


def test_product_seed_matches_oracle():
    """product_seed (src/apply.jl:655-685) on the host mirror equals the oracle's."""
    from kfgpu import circuits
    from kfgpu.operator import KronFreeOperator
    th = ocirc.three_mode_theta(np.random.default_rng(9))
    dims, terms = circuits.three_mode_leaf(th, ncut=3, n2=12, n3=9)

    class Shim(KronFreeOperator):          # the host-side methods only, no device handle
        def __init__(self, dims, terms):
            self.dims, self.terms, self.constant, self.N = dims, terms, 0.0, int(np.prod(dims))
            self._h = None

    S = Shim(dims, terms)
    Ho = ocirc.three_mode_operator(th, ncut=3, n2=12, n3=9)
    Xs, Xo = S.product_seed(7), Ho.product_seed(7)
    # the same product states up to the sign of each column
    assert np.allclose(np.abs(np.sum(Xs * Xo, axis=0)), 1.0, atol=1e-10)
