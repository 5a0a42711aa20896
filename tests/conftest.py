import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built libsculptgpu")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu():
    from dune_sculpt_gb300 import build as b

    b.build()
    from dune_sculpt_gb300 import sculpt

    sculpt.load()
    sms, major, minor = sculpt.device_info()
    assert major >= 10, f"needs a Blackwell GPU, got sm_{major}{minor}"
    return sculpt
