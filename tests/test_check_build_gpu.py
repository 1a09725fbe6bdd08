"""The bounds-recording build (-DKF_CHECK): kfgpu.build.build_library(check=True) compiles every
kernel with its index tests on (the plane-marching apply's nine sites 101-109: each slice, ring,
weight, table and output index; the batched leaf solver's 201-203: the element decode of its apply
and update, the leaf's blocks against the CTA's scratch; the TMA-fed Gram's 301-303: raw-slot reads,
operand-image stores, each tensor copy's box; each tested before the access, a failure recorded,
never trapped) into libkfgpu_check.so.  The plane-marching parity tests (every stencil shape against
the oracle and the full-size three-mode leaf), the Gram's pools and ragged row counts and the batched
solver's tests then run in a subprocess on that library (KF_LIB), and the session fails unless the
library is a KF_CHECK build and no bounds check failed (KF_CHECK_CLEAN, tests/conftest.py)."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_plane_marching_clean_under_kf_check(cuda):
    from kfgpu.build import build_library
    lib = build_library(check=True)
    env = dict(os.environ, KF_LIB=lib, KF_CHECK_CLEAN="1")
    r = subprocess.run([sys.executable, "-m", "pytest", "tests/test_apply_gpu.py", "tests/test_gram_tc_gpu.py",
                        "tests/test_batch_gpu.py", "-k", "marching or against_fp64 or ragged or batched", "-q",
                        "-p", "no:cacheprovider"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-2000:])
    assert "passed" in r.stdout
