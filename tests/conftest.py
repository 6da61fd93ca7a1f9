"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the built
library; everything else runs on the CPU."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libzccl_gpu.so")


class Golden:
    """tests/golden/golden.{json,npz}, written by tests/golden/make_golden.py
    from the reference codec."""

    def __init__(self):
        with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
            self.meta = json.load(f)
        self.arr = np.load(os.path.join(GOLDEN_DIR, "golden.npz"))
        self.cases = self.meta["cases"]

    def x(self, c):
        return self.arr[c["x"]]

    def y(self, c):
        return self.arr[c["y"]]

    def stream(self, c, which="s") -> bytes:
        return self.arr[f"{which}{c['i']}"].tobytes()


@pytest.fixture(scope="session")
def golden():
    return Golden()


@pytest.fixture(scope="session")
def port():
    from oracle import zoracle
    return zoracle.port()
