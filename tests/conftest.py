import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the library's kernels")
    config.addinivalue_line("markers", "slow: full-size workloads")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu():
    if not has_gpu():
        pytest.fail("GPU test collected on a machine without a GPU (run with -m 'not gpu')")
    from bvh_gb300 import build
    build.build_library()
    import torch
    torch.cuda.init()
    return torch
