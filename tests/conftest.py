"""Test configuration: the ``gpu`` marker and repository paths.

``-m "not gpu"`` runs on any machine (oracle pins, API, translator, C-ABI
exports); ``-m gpu`` needs a CUDA device and a built ``libxk.so``.
"""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for path in (ROOT, os.path.join(ROOT, "oracle")):
    if path not in sys.path:
        sys.path.insert(0, path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libxk.so")


@pytest.fixture(autouse=True)
def _no_tuning_cache(monkeypatch):
    """Tests time their own tuning runs: the persistent tuning cache is off
    unless a test points ``XK_TUNE_CACHE`` at a file of its own."""
    monkeypatch.setenv("XK_TUNE_CACHE", "off")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as fh:
        return json.load(fh)
