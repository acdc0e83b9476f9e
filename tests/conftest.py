import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="session")
def golden600():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "water600.npz")))


@pytest.fixture(scope="session")
def golden4095():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "water4095.npz")))


@pytest.fixture(scope="session")
def golden_mc():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "mc.npz")))


@pytest.fixture(scope="session")
def golden_mts600():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "mts_water600.npz")))


@pytest.fixture(scope="session")
def golden_go_hc():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "go_hc.npz")))


@pytest.fixture(scope="session")
def golden_bgo600():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "bgo600.npz")))


@pytest.fixture(scope="session")
def golden_chain():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "chain900.npz")))
