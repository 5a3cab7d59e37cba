import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def native():
    """Builds (if stale) and loads the native libraries."""
    import __graft_entry__

    __graft_entry__.build()
    import vren_gb300

    return vren_gb300.lib()


@pytest.fixture(scope="session")
def cuda(native):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")


@pytest.fixture(autouse=True)
def _no_device_error(request):
    """After every GPU test, the device error word must be clear."""
    yield
    if request.node.get_closest_marker("gpu") is not None:
        import torch

        if torch.cuda.is_available():
            import vren_gb300

            err = vren_gb300.device_error(clear=True)
            assert err == 0, f"device error word set: {err}"
