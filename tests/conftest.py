import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the batch autotuner's per-shape cache: keep the test session's choices out of the user's
# cache directory (the library reads this variable when it stores or first loads choices)
if "O3G_TUNE_CACHE" not in os.environ:
    import tempfile
    os.environ["O3G_TUNE_CACHE"] = os.path.join(tempfile.mkdtemp(prefix="o3g_tune_"), "batch_tune.txt")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU; calls the CUDA path through the C-ABI")


@pytest.fixture(scope="session")
def cuda():
    """The GPU tests run on a GB300 machine; without one they fail loudly instead of skipping."""
    import torch
    assert torch.cuda.is_available(), "GPU test collected on a machine without CUDA"
    major, minor = torch.cuda.get_device_capability(0)
    assert (major, minor) == (10, 3), "expected an sm_103 GPU, got sm_%d%d" % (major, minor)
    from omega3d_gb300 import _lib
    _lib.lib()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def built_lib():
    """libo3dgpu.so, built here if needed (nvcc cross-compiles without a GPU)."""
    from omega3d_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.lib()
