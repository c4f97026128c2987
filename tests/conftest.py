"""Shared test configuration.

``-m gpu`` tests need a CUDA device and the compiled ``osiris_gb300`` library; everything else
runs on the CPU (oracle against the golden fixtures, host logic, library symbol checks).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle as po
    po.build(with_ref=False)
    return po
