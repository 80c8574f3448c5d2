"""Shared pytest setup: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the in-tree liblbmx.so; every
other test runs on the CPU (oracle, host logic, library symbol table).
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "cuda-lbm_gb300"), os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built liblbmx.so")
