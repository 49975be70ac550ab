"""Image epilogue on the GPU (mbx_colorize / mbx_render_image) against the
oracle's restatement of the reference's render tool and its BMP fixtures.

Exactness: the kernel reproduces the reference's float and double operations;
its libm calls are correctly rounded (logf/powf) or tabulated from the host's
libm, so against the oracle on the same host every byte is expected to agree
except where the host's logf/powf themselves are not correctly rounded (a few
inputs in 10^4, and then only when the neighbouring palette entry is hit).
The byte tolerance below is that: at most one sample per pixel block moved to
an adjacent palette entry.
"""
import numpy as np
import pytest

import mbx
import oracle
import views
from conftest import bmp_rgb, color_kwargs, load_color_cases, load_color_fixture

pytestmark = pytest.mark.gpu

CASES = load_color_cases()


def _params(c):
    return mbx.ColorParams(supersample=c["ss"], **color_kwargs(c))


def _agree(a, b, frac=1e-3, maxdiff=3):
    d = np.abs(a.astype(int) - b.astype(int))
    assert d.max() <= maxdiff and np.mean(d > 0) <= frac, (int(d.max()), float(np.mean(d > 0)))
    return float(np.mean(d > 0))


@pytest.fixture(scope="module")
def be():
    b = mbx.create_compute_backend("cuda")
    yield b
    b.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_colorize_golden(be, name):
    c = CASES[name]
    values, aux, bmp = load_color_fixture(name, c)
    got = be.colorize(values, c["width"], c["height"], _params(c), aux=aux)
    want = oracle.colorize(values, c["width"], c["height"], c["ss"], aux=aux, **color_kwargs(c))
    assert np.array_equal(got, want), name
    _agree(got, bmp_rgb(bmp, c["width"], c["height"]))


@pytest.mark.parametrize("mapping", [mbx.MAP_LOG_POWER, mbx.MAP_DISTANCE, mbx.MAP_STRIPE, mbx.MAP_TRAP])
@pytest.mark.parametrize("shading", [mbx.SHADE_NONE, mbx.SHADE_RELIEF, mbx.SHADE_NORMAL_MAP, mbx.SHADE_DE_OVERLAY])
def test_colorize_wide_values(be, mapping, shading):
    """Log-uniform values up to 1e6 (deep-zoom escape counts), interior and empty samples."""
    rng = np.random.RandomState(11 + 4 * mapping + shading)
    w, h, ss = 160, 90, 2
    v = (10.0 ** rng.uniform(0, 6, (h * ss, w * ss)) - 1).astype(np.float32)
    v[rng.uniform(size=v.shape) < 0.05] = -2.0
    v[rng.uniform(size=v.shape) < 0.01] = -10.0
    if mapping == mbx.MAP_STRIPE:
        v = np.where(v >= 0, rng.uniform(0, 1, v.shape), v).astype(np.float32)
    aux = None
    if shading == mbx.SHADE_NORMAL_MAP:
        aux = rng.uniform(-np.pi, np.pi, v.shape).astype(np.float32)
    elif shading == mbx.SHADE_DE_OVERLAY:
        aux = (10.0 ** rng.uniform(-3, 2, v.shape)).astype(np.float32)
    kw = dict(mapping=mapping, shading=shading, density=60.0, light_az=2.3, light_el=0.55, relief_strength=1.7, de_k=1.5)
    got = be.colorize(v, w, h, mbx.ColorParams(supersample=ss, **kw), aux=aux)
    want = oracle.colorize(v, w, h, ss, aux=aux, **kw)
    _agree(got, want, frac=2e-3)
    ms, fb = be.last_color_stats()
    assert ms > 0 and fb <= 0.01 * v.size


def test_colorize_device_tensors(be):
    torch = pytest.importorskip("torch")
    c = CASES["plain_ss3"]
    values, _, _ = load_color_fixture("plain_ss3", c)
    dv = torch.from_numpy(values.copy()).cuda()
    out = be.colorize(dv, c["width"], c["height"], _params(c))
    assert out.is_cuda and out.dtype == torch.uint8
    host = be.colorize(values, c["width"], c["height"], _params(c))
    assert np.array_equal(out.cpu().numpy(), host)


@pytest.mark.parametrize("ss,shading,cm", [(1, mbx.SHADE_NONE, 0), (3, mbx.SHADE_RELIEF, 0), (3, mbx.SHADE_DE_OVERLAY, mbx.DE_OVERLAY)])
def test_render_image_matches_compute_then_colour(be, ss, shading, cm):
    v = dict(center_re="-0.74364388703715", center_im="0.13182590420533", scale="100000", max_iterations=3000)
    w, h = 96 * ss, 54 * ss
    p = mbx.ColorParams(supersample=ss, shading=shading)
    img = be.render_image(mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], w, h, v["max_iterations"], coloring_method=cm), p)
    req = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], w, h, v["max_iterations"], coloring_method=cm)
    assert be.compute_status(req) == mbx.OK, be.last_error()
    aux = req.normal if shading == mbx.SHADE_DE_OVERLAY else None
    assert np.array_equal(img, be.colorize(req.iterations, w // ss, h // ss, p, aux=aux))
    want = oracle.colorize(req.iterations, w // ss, h // ss, ss, aux=aux, mapping=0, shading=shading, density=60.0, light_az=2.3, light_el=0.55, relief_strength=1.0, de_k=1.5)
    _agree(img, want)


def test_render_image_deep_mixed(be):
    """A 1e-300 frame in the mixed form, coloured on the device: escape values ~9400."""
    v = views.deep_view(300)
    req = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], 480, 270, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED)
    img = be.render_image(req, mbx.ColorParams())
    ref = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], 480, 270, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED)
    assert be.compute_status(ref) == mbx.OK
    want = oracle.colorize(ref.iterations, 480, 270, 1)
    frac = _agree(img, want, frac=1e-3)
    print("\n[color] 1e-300 480x270: bytes differing from the oracle %.2e" % frac)


def test_invalid_color_requests(be):
    c = CASES["plain_ss1"]
    values, _, _ = load_color_fixture("plain_ss1", c)
    for bad in (dict(supersample=0), dict(mapping=7), dict(shading=9), dict(density=0.0)):
        with pytest.raises(RuntimeError):
            be.colorize(values, c["width"], c["height"], mbx.ColorParams(**bad))
    with pytest.raises(RuntimeError):  # overlay needs its buffer
        be.colorize(values, c["width"], c["height"], mbx.ColorParams(shading=mbx.SHADE_DE_OVERLAY))
    req = mbx.ComputeRequest("-0.75", "0.1", "10", 100, 60, 500)
    with pytest.raises(RuntimeError):  # 100 is not a multiple of 3
        be.render_image(req, mbx.ColorParams(supersample=3))
    with pytest.raises(RuntimeError):  # no overlay buffer requested
        be.render_image(mbx.ComputeRequest("-0.75", "0.1", "10", 96, 60, 500), mbx.ColorParams(shading=mbx.SHADE_DE_OVERLAY))


def test_render_image_normal_map_matches_reference_tool(be):
    """MANDEL_NORMAL=1 end to end: the renderer's normal-map angles (exact form)
    shaded on the device, against the oracle colouring the same buffers."""
    v = dict(center_re="-0.74364388703715", center_im="0.13182590420533", scale="100000", max_iterations=3000)
    ss = 2
    w, h = 96 * ss, 54 * ss
    p = mbx.ColorParams(supersample=ss, shading=mbx.SHADE_NORMAL_MAP, light_el=0.9)
    img = be.render_image(mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], w, h, v["max_iterations"], coloring_method=mbx.NORMAL_MAP), p)
    req = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], w, h, v["max_iterations"], coloring_method=mbx.NORMAL_MAP)
    assert be.compute_status(req) == mbx.OK, be.last_error()
    want = oracle.colorize(req.iterations, w // ss, h // ss, ss, aux=req.normal, mapping=0, shading=mbx.SHADE_NORMAL_MAP, density=60.0, light_az=2.3, light_el=0.9, relief_strength=1.0, de_k=1.5)
    _agree(img, want)
