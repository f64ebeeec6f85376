import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def load_golden(name):
    import numpy as np

    return np.load(os.path.join(GOLDEN, name))


def cost_scale(total, per_image):
    """What the FP32 error of a mean ML cost scales with: the larger of the mean and the mean
    magnitude of its per-image terms, which take either sign and can cancel in the mean (a
    relative test of a near-zero mean would fail on rounding alone)."""
    import numpy as np

    per = per_image.detach().abs().mean().item() if hasattr(per_image, "detach") else float(np.mean(np.abs(per_image)))
    return max(abs(float(total)), per)


@pytest.fixture(scope="session")
def pkg():
    """The product package, with its CUDA library built in-tree (no fallback)."""
    sys.path.insert(0, ROOT)
    lib = os.path.join(ROOT, "3dcovarestimation_gb300", "libcov3d_gb300.so")
    if not os.path.exists(lib):
        import __graft_entry__

        __graft_entry__.build()
    return importlib.import_module("3dcovarestimation_gb300")


@pytest.fixture(scope="session")
def dev():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
