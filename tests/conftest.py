import os
import sys

import pytest

# the oracle's OpenMP loops only pay off on large grids; test cases are small
os.environ.setdefault("OMP_NUM_THREADS", "1")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long-running CPU test")
