"""Shared fixtures.  Tests marked `gpu` need a GB300; everything else runs on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def lib():
    """libkite_gb300.so, built in-tree if needed."""
    from ahnum_gb300.build import build_library
    from ahnum_gb300 import native
    build_library()
    return native.load()


@pytest.fixture(scope="session")
def oracle_mod():
    """The CPU oracle (test infrastructure), built in-tree if needed."""
    from oracle import oracle
    oracle.build(ref=False)
    oracle.load()
    return oracle
