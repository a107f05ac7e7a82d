import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the libvkcuda.so kernels)")


@pytest.fixture(scope="session")
def ctx():
    """One device context for the GPU tests. The library must load and a device must open:
    a GPU test never falls back to anything else."""
    from verkehrt_gb300 import build as vbuild

    vbuild.build()
    import verkehrt_gb300 as vk

    c = vk.Context(0)
    yield c
    c.close()
