import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def golden_outputs():
    return np.load(os.path.join(GOLDEN, "ref_outputs_vw4.npz"))


@pytest.fixture(scope="session")
def golden_layouts():
    return np.load(os.path.join(GOLDEN, "ref_layouts.npz"))


@pytest.fixture(scope="session")
def fftset_lib():
    """The CUDA library; fails (does not skip) when it cannot be loaded."""
    import fftset_gb300
    return fftset_gb300


@pytest.fixture(scope="session")
def gpu_set(fftset_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    s = fftset_lib.FftSet()
    yield s
    s.close()
