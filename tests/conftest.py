"""Shared test setup: import paths, the `gpu` marker, and library handles."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "parallel-db-buffer-management_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs through libpbm.so")


@pytest.fixture(scope="session")
def orc():
    r = subprocess.run(["make", "-s", "-C", ORACLE, "-j4"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def pbm_mod():
    import pbm

    pbm.lib()
    return pbm


@pytest.fixture(scope="session")
def cuda(pbm_mod):
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.set_device(0)
    return torch
