import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA kernels through the C ABI")


@pytest.fixture(scope="session")
def wf():
    """The product package with libwfpt.so built in-tree."""
    from vulkanwavefrontpathtracer_gb300 import build
    build.build()
    import vulkanwavefrontpathtracer_gb300 as pkg
    pkg._lib.load()
    return pkg


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def dev():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return torch.device("cuda:0")


def random_rays(rng, n, lo=0.0, hi=1.0, tmax=10.0, tmin=0.0):
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, :3] = o
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r
