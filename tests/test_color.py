"""Image epilogue on the CPU: the oracle against the reference's own render
tool, the library's host parts (palette, gamma steps, BMP writer) against the
oracle, and the device colour math compiled for the host.

* tests/golden/color_*.bmp are BMP files written by the reference's render
  tool (src/tools/render.cpp) next to the values it coloured
  (tests/golden/make_color_golden.py); the oracle must reproduce every byte.
* The library's palette and its gamma step positions are built by host code
  the kernel only reads; they must equal the oracle's palette and the direct
  evaluation of render.cpp's gamma encode.
* tests/color_math_check.cpp runs the kernel's pair-of-floats log/pow on the
  host: every accepted result must be the correctly rounded float.
"""
import os
import platform
import subprocess
import tempfile

import numpy as np
import pytest

import mbx
import oracle
from conftest import ROOT, bmp_rgb, color_kwargs, load_color_cases, load_color_fixture

CASES = load_color_cases()
X86 = platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_reference_bmp(name):
    c = CASES[name]
    values, aux, bmp = load_color_fixture(name, c)
    rgb = oracle.colorize(values, c["width"], c["height"], c["ss"], aux=aux, **color_kwargs(c))
    out = oracle.bmp_bytes(rgb)
    if X86:
        assert out == bmp
    else:  # another libm: the palette's powf may round differently in the last place
        diff = np.abs(rgb.astype(int) - bmp_rgb(bmp, c["width"], c["height"]).astype(int))
        assert diff.max() <= 1 and np.mean(diff > 0) < 1e-3


def test_write_bmp_matches_reference_writer():
    for name in ("plain_ss1", "relief_ss2"):
        c = CASES[name]
        _, _, bmp = load_color_fixture(name, c)
        rgb = bmp_rgb(bmp, c["width"], c["height"])
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "x.bmp")
            mbx.write_bmp(path, rgb)
            with open(path, "rb") as f:
                assert f.read() == bmp
    # odd widths pad rows to four bytes
    rgb = np.arange(5 * 3 * 3, dtype=np.uint8).reshape(3, 5, 3)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "y.bmp")
        mbx.write_bmp(path, rgb)
        with open(path, "rb") as f:
            assert f.read() == oracle.bmp_bytes(rgb)


def test_palette_matches_oracle():
    pal, _ = mbx.color_tables()
    assert np.array_equal(pal.view(np.uint32), oracle.palette().view(np.uint32))


def _gamma_value(l):
    return oracle.gamma_value(l)


def test_gamma_steps_are_exact():
    _, thr = mbx.color_tables()
    assert np.all(np.diff(thr) > 0)
    k = np.arange(1, thr.size + 1)
    # each step is the first float reaching its value
    assert np.all(_gamma_value(thr) >= k)
    below = np.nextafter(thr, np.float32(-1))
    assert np.all(_gamma_value(below) < k)
    # monotone around every step and on random values: the table gives the encode
    win = (thr.view(np.int32)[:, None] + np.arange(-64, 65)[None, :]).astype(np.int32).view(np.float32).ravel()
    rnd = np.random.RandomState(3).uniform(0, 1.2, 1_000_000).astype(np.float32)
    for l in (win, rnd):
        assert np.array_equal(np.searchsorted(thr, l, side="right"), _gamma_value(l))


def test_device_math_rounds_correctly_on_host():
    src = os.path.join(ROOT, "tests", "color_math_check.cpp")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "cm")
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", src, "-o", exe])
        for density in ("60", "45", "200"):
            out = subprocess.check_output([exe, "2000000", density], text=True).split()
            n, bad_log, bad_pow, fb_log, fb_pow = (int(x) for x in out[:5])
            max_log, max_pow = float(out[5]), float(out[6])
            # accepted results are the correctly rounded floats
            assert bad_log == 0 and bad_pow == 0, density
            # the FP64 path stays rare; the pair errors sit inside the bounds the
            # rounding check assumes (log 2^-44; pow |y| 2^-44 + 2^-44, |y| < 20 here)
            assert fb_log + fb_pow < 5e-5 * n, density
            assert max_log < 2.0 ** -45 and max_pow < 21 * 2.0 ** -44, density


def test_color_params_validation_without_gpu():
    p = mbx.ColorParams(supersample=3, shading=mbx.SHADE_RELIEF)
    assert p.supersample == 3 and p.shading == 1 and abs(p.density - 60.0) < 1e-6
    with pytest.raises(TypeError):
        mbx.ColorParams(bogus=1)
