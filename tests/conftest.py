import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the GB300 kernels)")


@pytest.fixture(scope="session")
def small_cfg():
    """The small phantom at 48^3 (2.67 mm voxels), 48x48 image: oracle-sized."""
    from volview_gb300 import scene
    return scene.small_config(n=48, size=48, spp=4)


@pytest.fixture(scope="session")
def gpu_ctx():
    from volview_gb300 import renderer as R
    ctx = R.Context(0)
    yield ctx
    ctx.destroy()
