import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdcf_gb300.so")
    config.addinivalue_line("markers", "reference: needs the reference checkout to compile the reference oracle")


@pytest.fixture(scope="session")
def lena():
    return np.load(os.path.join(GOLDEN, "lena_fixtures.npz"))


@pytest.fixture(scope="session")
def synthetic():
    z = np.load(os.path.join(GOLDEN, "synthetic_reference.npz"))
    cases = {}
    for key in z.files:
        name, field = key.split("/", 1)
        cases.setdefault(name, {})[field] = z[key]
    return cases


@pytest.fixture(scope="session")
def port_lib():
    from oracle import oracle
    oracle.build(ref=False)
    return oracle


@pytest.fixture(scope="session")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import disccofan_gb300 as dcf
    return dcf.Context(0)
