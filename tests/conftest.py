"""Test configuration: the `gpu` marker and import paths (package root and the oracle)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU and the built libgbp.so")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_prop():
    from scip_gb300 import gbp
    from scip_gb300.build import build_libgbp

    build_libgbp()
    p = gbp.Propagator(0)
    yield p
    p.close()
