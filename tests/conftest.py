import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "sedona-db_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build(with_ref=False)
    return oracle


def pytest_collection_modifyitems(config, items):
    # GPU tests are only run when asked for with -m gpu; without a GPU they
    # would fail loudly by design (the product has no CPU fallback).
    pass
