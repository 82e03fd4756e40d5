import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "highvoronoi.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libhvgpu.so")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds libhvgpu and returns the package; fails (never skips) without a GPU."""
    import __graft_entry__ as g
    g.build()
    import hvgpu
    hvgpu.default_context()
    return hvgpu
