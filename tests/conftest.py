"""Shared fixtures; registers the ``gpu`` marker."""
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


@pytest.fixture(scope="session")
def golden():
    """The 2113-node plate fixture (inputs and expected outputs)."""
    return dict(np.load(GOLDEN / "plate2113.npz"))


@pytest.fixture(scope="session")
def plate(golden):
    """Inputs of the reference regression setup, built from the fixture."""
    from tests.plate_setup import plate_inputs
    return plate_inputs(golden)
