import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)



def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path through the C-ABI)")
    config.addinivalue_line("markers", "slow: full-size GPU-scale case")
    # build the library and the oracle if this checkout has not been built yet
    from twoscalerich_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    if not os.path.exists(os.path.join(ROOT, "oracle", "libtsr_oracle.so")):
        B.build_oracle()


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    from twoscalerich_gb300 import capi
    return capi.load()


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.load()
