import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")
# The reference checkout, for the tests that read its sources or data where
# it exists: ASDPOCS_REFERENCE_DIR, else a checkout named "reference" beside
# the repository.
REFERENCE = os.environ.get("ASDPOCS_REFERENCE_DIR") or os.path.join(
    os.path.dirname(ROOT), "reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def lib():
    """The product library, built in-tree if needed."""
    from asd_pocs_mex_cuda_demo_gb300 import build

    build.build()
    import asd_pocs_mex_cuda_demo_gb300 as pkg

    return pkg.load()


@pytest.fixture(scope="session")
def gpu(lib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))
