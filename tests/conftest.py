"""Shared pytest setup.

* registers the `gpu` marker (tests that need a GB300; everything else runs
  on CPU);
* puts the repo root (for `oracle`) and openmp-blas_gb300/ (for `gbblas`) on
  sys.path;
* builds the CPU oracle once per session.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "openmp-blas_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
    yield


@pytest.fixture(scope="session")
def cuda():
    """torch with a visible sm_103 device, or a loud failure."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    cap = torch.cuda.get_device_capability(0)
    if cap != (10, 3):
        pytest.fail(f"expected an sm_103 (GB300) device, found sm_{cap[0]}{cap[1]}")
    import gbblas
    gbblas.lib()
    return torch
