import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the reference tree for the tests that read its own golden data
# (TOASTPP_REFERENCE; those tests skip where it is absent)
REFERENCE = os.environ.get("TOASTPP_REFERENCE", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libtoastgpu.so")


def has_reference():
    return os.path.isdir(os.path.join(REFERENCE, "test"))


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle
