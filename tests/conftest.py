import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA engine")


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import build
    if not build.reference_available():
        pytest.skip("reference tree absent: the reference-built oracle is only available where it is")
    from oracle.pyoracle import Reference
    return Reference()


@pytest.fixture(scope="session")
def tangent():
    from oracle.pyoracle import Tangent
    return Tangent()
