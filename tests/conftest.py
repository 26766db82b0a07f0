import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ORACLE = os.path.join(ROOT, "oracle")
if ORACLE not in sys.path:
    sys.path.insert(0, ORACLE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels through the C ABI)")
    config.addinivalue_line("markers", "slow: long-running CPU check")


def close(a, b, digits):
    """vitest's toBeCloseTo(b, digits): |a - b| < 10^-digits / 2."""
    return abs(a - b) < 10 ** (-digits) / 2
