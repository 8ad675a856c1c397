"""Shared fixtures: import paths, the `gpu` marker, and the built libraries."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "web-gs-renderer_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libwebgs.so)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Builds libwebgs.so and the oracle library once per session (incremental); with WEBGS_CHECKED=1
    also the checked build, which the tests then load instead of the product library."""
    import os

    from build import build_all  # web-gs-renderer_gb300/build.py

    build_all(checked=os.environ.get("WEBGS_CHECKED") == "1")
    yield


@pytest.fixture(scope="session")
def gpu_ctx():
    """A default context (16x16 tiles, 8-bit digits, batch 256, factor 64) shared by GPU tests."""
    import webgs

    ctx = webgs.Context()
    yield ctx
    ctx.close()
