import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libmcbound.so")
    config.addinivalue_line("markers", "slow: long CPU run (minutes)")
    # temporary files of the tests stay inside the repository (git-ignored)
    if not config.option.basetemp:
        config.option.basetemp = os.path.join(ROOT, ".pytest_tmp")


def has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    from madam_gb300 import lib as M

    if not os.path.exists(M.LIB_PATH):
        from madam_gb300 import build as B

        B.build()
    return M


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O

    O.lib()
    return O
