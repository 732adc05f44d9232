import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def renderer():
    """A Renderer on cuda:0 over the freshly built library (fails loudly when
    the library cannot be built or loaded)."""
    from blackhole_8_gb300 import build
    build.build()
    from blackhole_8_gb300.render import Renderer
    r = Renderer(0)
    yield r
    r.close()
