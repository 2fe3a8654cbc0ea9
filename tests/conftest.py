"""Shared test setup: import paths for the gbcompute binding and the CPU
oracle, the `gpu` marker, and a session-wide context for GPU tests."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "opencl-sdk_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbcompute.so")


@pytest.fixture(scope="session")
def gbc():
    import gbcompute

    return gbcompute


@pytest.fixture(scope="session")
def ctx(gbc):
    if gbc.device_count() == 0:
        pytest.fail("gpu test selected but no CUDA device is visible")
    c = gbc.Context()
    yield c
    c.close()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build()
    return oracle
