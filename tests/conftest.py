import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def hodlr():
    """The CUDA library on a real GPU.  No fallback: a GPU test fails if the
    library does not load."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastsolver2_gb300 as fs
    fs.lib(build_if_missing=True)
    return fs
