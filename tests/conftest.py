import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Native parts built in-tree (CUDA library, generators, oracle)."""
    from openph_gb300 import _build
    import oracle
    _build.build_gen()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def cuda_lib(built):
    from openph_gb300 import _build, api
    _build.build_cuda()
    return api.lib()


@pytest.fixture(scope="session")
def ctx(cuda_lib):
    from openph_gb300.api import Context
    c = Context(0)
    yield c
    c.close()
