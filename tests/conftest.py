"""Shared test setup: import paths, the `gpu` marker and fixture loaders."""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
for sub in ("centrex-tlf_gb300", "oracle", "tests/golden"):
    path = str(REPO / sub)
    if path not in sys.path:
        sys.path.insert(0, path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def golden():
    import codec

    cache = {}

    def load(name):
        if name not in cache:
            cache[name] = codec.load(name)
        return cache[name]

    return load
