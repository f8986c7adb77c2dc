import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build_oracle
    from oracle.oracle import Oracle

    build_oracle.build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import build_oracle
    from oracle.oracle import Reference

    if not build_oracle.build_reference():
        pytest.skip("reference sources not available on this machine")
    return Reference()


@pytest.fixture(scope="session")
def nsg():
    """The built libnsg module (builds it when missing)."""
    import nsphere_gb300 as ns
    from nsphere_gb300 import build as nbuild

    nbuild.build()
    ns.lib()
    return ns


def golden(name):
    return np.load(os.path.join(GOLDEN, name))
