import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "pixel-art-remaster-gpu_gb300"):
    p = os.path.join(REPO, sub)
    if p not in sys.path:
        sys.path.insert(0, p)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; calls the CUDA library through its C ABI")


@pytest.fixture(scope="session")
def cuda():
    """torch with a visible GPU and the library built; skips without a GPU."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import build as depix_build
    depix_build.build()
    import depix
    depix.lib()
    depix.init_device()
    return torch
