import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def port():
    import oracle

    return oracle.Port()


@pytest.fixture(scope="session")
def ctx():
    import poisson_caustic_design_gb300 as pcd

    c = pcd.Context(0)
    yield c
    c.close()


def solver_case_names():
    z = load_golden("solver_cases.npz")
    return sorted({k.split("/")[0] for k in z.files})
