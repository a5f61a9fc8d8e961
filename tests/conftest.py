import json
import os
import sys

import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(TESTS)
for p in (REPO, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle, build_oracle
    build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(TESTS, "golden", "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def native():
    """The product library, built in-tree; fails (never skips) when missing."""
    from sdhash_gb300 import build
    build.build_all()
    import sdhash_gb300
    return sdhash_gb300.lib()


@pytest.fixture(scope="session")
def ctx(native):
    import sdhash_gb300
    return sdhash_gb300.Context(int(os.environ.get("SDBFG_DEVICE", "0")))
