import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libgbompl.so")


@pytest.fixture(scope="session")
def port():
    from oracle.oracle import Oracle
    return Oracle.port()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    cache = {}

    def load(name):
        if name not in cache:
            with np.load(os.path.join(ROOT, "tests", "golden", f"{name}.npz")) as z:
                cache[name] = {k: z[k] for k in z.files}
        return cache[name]
    return load
