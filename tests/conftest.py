"""Shared fixtures.  `gpu`-marked tests need a CUDA device and call the
library through its C ABI; everything else runs on the CPU."""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ORACLE_DIR = os.path.join(ROOT, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the CUDA library")


@pytest.fixture(scope="session")
def ckm():
    """The package (cl-kmeans_gb300) with libckm.so loaded."""
    mod = importlib.import_module("cl-kmeans_gb300")
    if not os.path.exists(mod.LIB_PATH):
        mod.build()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu-marked tests")
    return torch.device("cuda:0")


def blobs(n, d, k_blobs, seed, spread=10.0, sigma=1.0):
    """Seeded Gaussian blobs, returned as the flat column-major float32
    array P[f * n + p] (the reference layout)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-spread, spread, size=(k_blobs, d))
    comp = rng.integers(0, k_blobs, size=n)
    X = centres[comp] + sigma * rng.standard_normal((n, d))
    return np.ascontiguousarray(X.astype(np.float32).T).reshape(-1)
