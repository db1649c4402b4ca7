import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib():
    from flag4j_gb300 import build
    build.build()
    from flag4j_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def f4j(lib):
    import flag4j_gb300
    return flag4j_gb300


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_golden.json")) as fh:
        return json.load(fh)


U = 2.0 ** -53


def assert_within_bound(C, ref, absab, k, what=""):
    """Componentwise |C - C_ref| <= 2 k u |A||B| (u = 2^-53, k = inner dimension)."""
    import numpy as np
    bound = 2.0 * max(k, 1) * U * absab
    err = np.abs(C - ref)
    bad = err > bound
    assert not np.any(bad), "%s: %d entries outside 2ku|A||B|, worst excess %g" % (
        what, int(bad.sum()), float((err - bound)[bad].max()))
