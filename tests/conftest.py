import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def background():
    from imgutil import golden_image
    return golden_image("background.png")


@pytest.fixture(scope="session")
def foreground():
    from imgutil import golden_image
    return golden_image("foreground.png")


@pytest.fixture(scope="session")
def goldens():
    from imgutil import golden_hashes
    return golden_hashes()
