import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) and the built CUDA library")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build()  # _ref/libref.so too where a reference checkout is named
    return oracle


def golden(name):
    import numpy as np

    return np.load(os.path.join(REPO, "tests", "golden", name))
