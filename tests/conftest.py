import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libbhk.so")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle as po
    if not os.path.exists(po.LIB_ORACLE):
        po.build()
    return po.Oracle()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name)))
    return load


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from black_simulation_gb300 import build
    build.build()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def ctx(cuda):
    from black_simulation_gb300 import bhk
    c = bhk.Context(0)
    yield c
    c.close()
