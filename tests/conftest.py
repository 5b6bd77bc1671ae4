import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built libgp_ptp.so")


def golden_cases():
    """(name, npz) of every committed golden fixture."""
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        out.append((os.path.splitext(os.path.basename(p))[0], dict(np.load(p))))
    return out


@pytest.fixture(scope="session")
def built_lib():
    from gproshan_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def gpu_ctx(built_lib):
    from gproshan_gb300 import _capi
    return _capi.Context(0)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle
