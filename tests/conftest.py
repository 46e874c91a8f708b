import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden_testdata():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "reference_testdata.npz")))


@pytest.fixture(scope="session")
def golden_synth():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "reference_synth.npz")))


@pytest.fixture(scope="session")
def golden_traversals():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "reference_traversals.npz")))
