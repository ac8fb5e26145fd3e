import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libfsi_gpu.so")
    config.addinivalue_line("markers", "slow: full-size acceptance runs (minutes of oracle time on the host)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads libfsi_gpu.so; there is no CPU fallback."""
    import fsilbm3d_gb300.build as b
    b.build()
    import fsilbm3d_gb300 as F
    return F.load_library()
