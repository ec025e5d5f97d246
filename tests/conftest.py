import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the CPU oracle and the library once per session (cheap if fresh)."""
    from oracle import oracle as O
    O.build(ref=False)
    import nbody_gb300.build as B
    B.build()


def golden(name: str):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


GOLDEN_FORCE_CASES = ["ball2048", "refic1024_seed7", "plummer4096", "ragged1000"]


def have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    major, minor = torch.cuda.get_device_capability(0)
    if (major, minor) != (10, 3):
        pytest.fail(f"expected an sm_103 (GB300) device, found sm_{major}{minor}")
    return torch.device("cuda:0")
