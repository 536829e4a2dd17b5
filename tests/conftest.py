"""Shared test setup: import paths, the `gpu` marker, built libraries."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "ewfa-gpu_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Compile libwfe and the oracle once per session (no-ops when up to date)."""
    import build as wfe_build  # ewfa-gpu_gb300/build.py
    import oracle

    wfe_build.build()
    oracle.build(ref=False)
    yield
