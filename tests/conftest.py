import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "parallel-si_gb300")
for p in (ROOT, PKG, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def pytest_collection_modifyitems(config, items):
    # keep the GPU tests of a file after its CPU tests
    items.sort(key=lambda it: (it.fspath.basename, 1 if it.get_closest_marker("gpu") else 0))
