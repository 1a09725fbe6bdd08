import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "kronfreecircuits.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libkfgpu.so")


def pytest_sessionfinish(session, exitstatus):
    """With KF_CHECK_CLEAN=1 (a run against the bounds-recording library, KF_LIB): fail the session
    when the library is not a KF_CHECK build or a kernel recorded a failed bounds check."""
    if os.environ.get("KF_CHECK_CLEAN") != "1":
        return
    import ctypes as C
    from kfgpu import _abi
    site, chk = C.c_int32(0), C.c_int32(0)
    _abi.check(_abi.lib().kf_test_check_word(C.byref(site), C.byref(chk)))
    if chk.value != 1 or site.value != 0:
        print(f"\nKF_CHECK: check build {chk.value}, first failed bounds-check site {site.value}")
        session.exitstatus = 1


@pytest.fixture(scope="session")
def goldens():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_goldens.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def cuda():
    """Skip-free guard: a GPU test without a GPU fails loudly instead of silently passing."""
    import torch
    assert torch.cuda.is_available(), "this test needs a CUDA device"
    from kfgpu.build import build_library
    build_library()
    torch.zeros(1, device="cuda")
    return torch
