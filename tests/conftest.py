import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "coolpdlp.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library (built on demand); GPU tests fail loudly without it."""
    from coolpdlp import build as B
    B.build_library()
    from coolpdlp import _abi
    return _abi.load_library()


@pytest.fixture(scope="session")
def handle(cuda_lib):
    from coolpdlp import native
    return native.default_handle(0)
