import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, ROOT, os.path.join(ROOT, "bayesian-turbulence-modeling_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")


@pytest.fixture(autouse=True)
def _seeded_rng():
    # deterministic tests (tests/python/conftest.py of the reference seeds the same way)
    np.random.seed(0)
    yield


@pytest.fixture(scope="session")
def oracle():
    from oracle import port
    port.build()
    return port
