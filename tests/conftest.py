import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


def reference_root():
    """The Wannier90 source tree the fixture scripts and the reference-file tests read:
    the W90_REFERENCE environment variable, or None (those tests skip)."""
    r = os.environ.get("W90_REFERENCE")
    return r if r and os.path.isdir(r) else None
