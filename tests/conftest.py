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
