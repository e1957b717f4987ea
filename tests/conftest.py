"""Shared fixtures.  Tests marked `gpu` need a CUDA device (a GB300); the
rest run on any machine (the CPU suite: oracle vs golden fixtures, the device
API under the host lane emulator, C ABI exports and argument checks)."""
import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def golden_cases():
    with open(GOLDEN / "golden.json") as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="session")
def golden_arrays():
    import numpy as np
    return dict(np.load(GOLDEN / "transposes.npz"))


@pytest.fixture(scope="session")
def trove_lib():
    """The CUDA library, built if stale (the build needs only nvcc)."""
    import trove_gb300
    from trove_gb300 import _build
    _build.build()
    return trove_gb300.load()


@pytest.fixture(scope="session")
def cuda(trove_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
