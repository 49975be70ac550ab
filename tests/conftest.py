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


def load_color_cases():
    with open(os.path.join(GOLDEN, "color_cases.json")) as f:
        return json.load(f)


def load_color_fixture(name, case):
    """(values, aux or None, reference BMP bytes) of an image-epilogue case."""
    n = case["width"] * case["height"] * case["ss"] ** 2
    a = np.fromfile(os.path.join(GOLDEN, "color_%s.f32" % name), dtype="<f4")
    with open(os.path.join(GOLDEN, "color_%s.bmp" % name), "rb") as f:
        bmp = f.read()
    return a[:n], (a[n:] if a.size > n else None), bmp


def bmp_rgb(bmp, width, height):
    """RGB [height][width][3] of a bottom-up 24-bit BMP."""
    row = (width * 3 + 3) & ~3
    data = np.frombuffer(bmp, np.uint8, offset=54).reshape(height, row)[::-1, : width * 3]
    return data.reshape(height, width, 3)[:, :, ::-1].copy()


def color_kwargs(case):
    return {k: case[k] for k in ("mapping", "shading", "density", "light_az", "light_el", "relief_strength", "de_k")}


def load_julia_cases():
    with open(os.path.join(GOLDEN, "julia_cases.json")) as f:
        return json.load(f)


def load_julia_fixture(name):
    """The reference engine's Mandel::ComputeJulia output for a case (float32)."""
    return np.fromfile(os.path.join(GOLDEN, "ref_julia_%s.f32" % name), dtype="<f4")


def load_truth(label):
    """(idx, N, value) of a 1080p frame's committed arbitrary-precision truth
    subset (tests/golden/make_truth.py), or None when it has not been made."""
    p = os.path.join(GOLDEN, "truth_c2_%s.npz" % label)
    if not os.path.exists(p):
        return None
    z = np.load(p)
    return z["idx"], z["N"], z["value"]
