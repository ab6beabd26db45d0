import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libftgpu.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as orc
    if not os.path.exists(orc.LIB):
        orc.build()
    return orc


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return {k: np.load(os.path.join(GOLDEN, k + ".npz")) for k in ("ref_force", "ref_ex9", "ref_cube",
                                                                 "ref_rigid")}


@pytest.fixture(scope="session")
def golden_reader():
    import numpy as np
    return np.load(os.path.join(GOLDEN, "ref_reader.npz"))
