"""Shared fixtures. Tests marked ``gpu`` need a CUDA device and the built
library; everything else runs on the CPU (oracle vs golden fixtures, host
logic, C-ABI symbol checks)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libaxs_gb300.so")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def axs():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import axion_strings_adaptive_gb300 as A
    A.build()
    A.lib()
    return A
