import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS, os.path.join(TESTS, "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built library")


@pytest.fixture(scope="session")
def small_tables():
    """Synthetic tables with the small xillver grid (written once per checkout)."""
    from relxill_gb300 import synth_tables

    d = os.path.join(ROOT, "_tables", "small")
    synth_tables.ensure_tables(d, xill="small")
    os.environ["RELXILL_TABLE_PATH"] = d
    return d


@pytest.fixture(scope="session")
def oracle(small_tables):
    import oracle_lib

    return oracle_lib.lib(small_tables)


@pytest.fixture(scope="session")
def gpu(small_tables):
    import relxill_gb300 as R

    R.init(small_tables)
    return R
