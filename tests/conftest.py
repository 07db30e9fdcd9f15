import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def synth_lib():
    from nav24_gb300.build import build_synth
    return build_synth()


@pytest.fixture(scope="session")
def product_lib():
    from nav24_gb300.build import build_product
    return build_product()


@pytest.fixture(scope="session")
def ctx(product_lib):
    from nav24_gb300 import Context
    c = Context(0)
    yield c
    c.close()
