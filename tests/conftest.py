import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "codim-ipc_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import build_lib
    build_lib.build()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle_ffi
    oracle_ffi.lib()
    return oracle_ffi
