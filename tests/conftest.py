"""Shared test set-up: the `gpu` marker, import path, on-demand builds."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Build libfivonagi.so and the oracle if a previous build() did not."""
    from fivonagi_gb300 import _abi, build
    from oracle import oracle
    if not os.path.exists(_abi.LIB_PATH):
        build.build()
    if not os.path.exists(oracle.ORACLE_LIB):
        oracle.build_oracle(with_ref=False)
    yield
