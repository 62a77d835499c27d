import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "randomballcover-gpu_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (os.path.join(ROOT, "oracle"), PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def engine_lib():
    import build_ext
    build_ext.build()
    import pyrbc
    pyrbc.lib()
    return pyrbc


@pytest.fixture(scope="session")
def rbc(engine_lib):
    """The engine on a real GPU (gpu-marked tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA GPU is required for gpu-marked tests")
    return engine_lib


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def sample_inputs():
    X = np.fromfile(os.path.join(GOLDEN, "sample_db.bin"), np.float32).reshape(1024, 16)
    Q = np.fromfile(os.path.join(GOLDEN, "sample_queries.bin"), np.float32).reshape(128, 16)
    return X, Q
