import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: larger CPU cases")


@pytest.fixture(scope="session")
def gpu_context():
    import mray_gb300 as M

    import torch

    ctx = M.Context(0)
    # torch's current (default) stream: the tests' tensor fills and copies are ordered with the library's kernels
    ctx.set_stream(torch.cuda.current_stream())
    yield ctx
    ctx.close()
