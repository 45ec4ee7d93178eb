import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path)")


@pytest.fixture(scope="session")
def gpu():
    """The native library on cuda:0.  A GPU test that cannot get it fails: on a
    machine with a GB300 a skip would hide a broken build."""
    import fritillaria_gb300 as frt

    frt.lib()
    if not frt.cuda_is_usable():
        pytest.fail("no usable GB300: the CUDA path cannot run")
    return frt
