import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gpu_lib():
    """The built library with tables uploaded (D3D10 default decoder)."""
    import torch

    import icbc_gb300 as ig
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ig.load()
    ig.init(ig.Decoder_D3D10)
    return ig
