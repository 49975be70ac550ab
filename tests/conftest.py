import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mandelbrot-explorer_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def load_cases():
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        return json.load(f)


def load_fixture(name, case):
    n = case["width"] * case["height"] * case["sub"] ** 2
    a = np.fromfile(os.path.join(GOLDEN, "ref_%s.f32" % name), dtype="<f4")
    it = a[:n]
    nr = a[n:] if a.size > n else None
    return it, nr


@pytest.fixture(scope="session")
def cases():
    return load_cases()
