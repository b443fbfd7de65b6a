"""Shared fixtures. `-m gpu` tests need a CUDA device and the native library; the rest run on CPU."""
import importlib
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "bigwave_golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and librs_fresnel.so")


@pytest.fixture(scope="session")
def rs():
    return importlib.import_module("3d_ravesim_gb300")


@pytest.fixture(scope="session")
def oracle():
    from oracle import bigwave_oracle
    return bigwave_oracle


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def cuda(rs):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    rs.build()
    rs._lib.lib()
    return torch.device("cuda", 0)


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), np.finfo(float).eps))
