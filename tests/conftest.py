import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the CUDA library")


@pytest.fixture(scope="session")
def pkg():
    return graft.load_package()


@pytest.fixture(scope="session")
def oracle():
    orc = graft.load_oracle()
    orc.build(ref=None)
    return orc


@pytest.fixture(scope="session")
def lib(pkg):
    """The CUDA library; built here if missing (the product never falls back)."""
    if not pkg.LIB_PATH.exists():
        pkg.build()
    return pkg.lib()


@pytest.fixture(scope="session")
def cuda(lib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    torch.cuda.set_device(0)
    return torch


def golden(name):
    d = np.load(GOLDEN / f"{name}.npz", allow_pickle=False)
    return {k: d[k] for k in d.files}


class GoldenCsr:
    def __init__(self, d):
        self.ptr, self.col, self.val = d["ptr"], d["col"], d["val"]

    @property
    def n(self):
        return int(self.ptr.shape[0] - 1)

    @property
    def nnz(self):
        return int(self.ptr[-1])
