"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "genfft_ref_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def golden():
    """Golden vectors produced by the reference genFFT (tests/golden/make_golden.py)."""
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gfft():
    """The product library on a GPU; fails (not skips) when it cannot load."""
    import torch
    assert torch.cuda.is_available(), "GPU test without a CUDA device"
    import genfft_gb300 as G
    if not os.path.exists(G.lib_path()):
        from genfft_gb300 import build
        build.build()
    G.lib()
    return G
