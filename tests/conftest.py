"""Test configuration: the `gpu` marker and the in-tree build."""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the native libraries in-tree if they are missing or stale."""
    from raycer_gb300 import build

    build.build_all()
    yield
