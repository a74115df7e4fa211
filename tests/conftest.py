import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_libs():
    """Builds the oracle and the scene generators (CPU) once per session."""
    from mray_gb300 import build as B
    import oracle.build as OB
    B.build_scenes()
    OB.build_oracle()
    return True


@pytest.fixture(scope="session")
def cuda_lib():
    """Builds libmray_gb300.so (nvcc cross-compiles without a GPU)."""
    from mray_gb300 import build as B
    B.build()
    return B.LIB
