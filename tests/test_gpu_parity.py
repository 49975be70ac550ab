"""CUDA renderer (exact form) against the oracle and the reference fixtures.

Bar: class (interior / exterior / empty) and escape iteration N identical for
every sample; smooth value / distance within 1e-6 relative (the only allowed
difference is the last-ulp behaviour of log on the GPU vs the host libm).
"""
import numpy as np
import pytest

import mbx
import oracle
from conftest import load_cases, load_fixture

CASES = load_cases()
pytestmark = pytest.mark.gpu
RTOL = 1e-6


@pytest.fixture(scope="module")
def backend():
    be = mbx.create_compute_backend("cuda")
    yield be
    be.close()


def gpu_render(be, c, **kw):
    req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"], sub=c["sub"], coloring_method=c["coloring_method"], bailout=c["bailout"], **kw)
    rc = be.compute_status(req)
    assert rc == mbx.OK, be.last_error()
    return req.iterations, req.normal, req.escape_iteration, be.last_stats.as_dict()


def assert_same(it, en, ref_it, ref_en, label):
    assert np.array_equal(it == -10.0, ref_it == -10.0), label + ": empty samples differ"
    assert np.array_equal(it < -1.5, ref_it < -1.5), label + ": interior/exterior class differs"
    if ref_en is not None:
        mism = np.nonzero(en != ref_en)[0]
        assert mism.size == 0, "%s: escape iteration differs at %d samples, first %s" % (label, mism.size, [(int(i), int(en[i]), int(ref_en[i])) for i in mism[:5]])
    np.testing.assert_allclose(it, ref_it, rtol=RTOL, atol=0, err_msg=label)


@pytest.mark.parametrize("name", sorted(CASES))
def test_exact_matches_oracle(backend, name):
    c = CASES[name]
    it, nr, en, st = gpu_render(backend, c)
    oit, onr, oen, ost = oracle.render(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"], sub=c["sub"], coloring_method=c["coloring_method"], bailout=c["bailout"])
    assert_same(it, en, oit, oen, name)
    if c["coloring_method"] & (16 | 64):
        np.testing.assert_allclose(nr, onr, rtol=RTOL, atol=0)
    assert st["kernel_launches"] > 0 and st["samples"] > 0


@pytest.mark.parametrize("name", sorted(CASES))
def test_exact_matches_reference_fixture(backend, name):
    c = CASES[name]
    it, nr, en, _ = gpu_render(backend, c)
    ref_it, ref_nr = load_fixture(name, c)
    assert_same(it, en, ref_it, None, name)
    if ref_nr is not None:
        np.testing.assert_allclose(nr, ref_nr, rtol=RTOL, atol=0)


def test_c1_config_matches_oracle(backend):
    """The plain FP64 configuration as stated: the seahorse-valley centre
    extended to 120 seed-drawn digits, 1280x720, half-width 1e-30, maxiter
    50000, bailout 2^8, through mbx_compute in the exact form against the
    oracle's restatement of the reference's double delta loop
    (mp.cpp:2290-2585): class and N identical at every sample, value within
    1e-6 relative."""
    import views

    v = views.c1_view()
    c = dict(v, width=1280, height=720, sub=1, coloring_method=0)
    it, _, en, st = gpu_render(backend, c, precision_mode=mbx.PRECISION_EXACT)
    assert st["used_floatexp"] == 0  # scale 2e30 stays on the double path
    oit, _, oen, _ = oracle.render(v["center_re"], v["center_im"], v["scale"], 1280, 720, v["max_iterations"], bailout=v["bailout"])
    assert_same(it, en, oit, oen, "c1 1280x720")
    print("\n[c1 1280x720] %d samples identical in class and N; N %d..%d" % (en.size, int(en[en > 0].min(initial=0)), int(en.max())))


def test_repeat_is_deterministic(backend):
    c = CASES["flake"]
    a = gpu_render(backend, c)[0]
    b = gpu_render(backend, c)[0]
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_device_outputs(backend):
    torch = pytest.importorskip("torch")
    c = CASES["minibrot875"]
    n = c["width"] * c["height"]
    it = torch.empty(n, dtype=torch.float32, device="cuda")
    en = torch.empty(n, dtype=torch.int32, device="cuda")
    req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"], bailout=c["bailout"], iterations=it, escape_iteration=en)
    assert backend.compute_status(req) == mbx.OK, backend.last_error()
    host_it, _, host_en, _ = gpu_render(backend, c)
    assert np.array_equal(it.cpu().numpy().view(np.uint32), host_it.view(np.uint32))
    assert np.array_equal(en.cpu().numpy(), host_en)


def test_invalid_requests_rejected(backend):
    c = CASES["c1"]
    for bad in (dict(sub=2), dict(width=1), dict(max_iterations=0), dict(coloring_method=128), dict(row_base=5)):
        kw = dict(sub=1)
        kw.update(bad)
        req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], kw.pop("width", 16), 9, kw.pop("max_iterations", 100), **kw)
        assert backend.compute_status(req) == mbx.E_INVALID
    req = mbx.ComputeRequest("x", "0", "100", 16, 9, 100)
    assert backend.compute_status(req) == mbx.E_INVALID


def test_strip_render_matches_oracle_strips(backend):
    """Strip export (full_height/row_base, mp.cpp:1399-1424): each strip equals
    the oracle's strip render exactly and the full frame to within rounding of
    the shifted origin (the reference's MANDEL_STRIPS validation)."""
    c = dict(CASES["shallow"])
    full = gpu_render(backend, c)[0].reshape(c["height"], c["width"])
    sh = 32
    for base in range(0, c["height"], sh):
        h = min(sh, c["height"] - base)
        req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], h, c["max_iterations"], bailout=c["bailout"], full_height=c["height"], row_base=base)
        assert backend.compute_status(req) == mbx.OK
        oit, _, oen, _ = oracle.render(c["center_re"], c["center_im"], c["scale"], c["width"], h, c["max_iterations"], bailout=c["bailout"], full_height=c["height"], row_base=base)
        assert_same(req.iterations, req.escape_iteration, oit, oen, "strip %d" % base)
        np.testing.assert_allclose(req.iterations.reshape(h, c["width"]), full[base : base + h], rtol=1e-5)


def test_orbit_colourings_take_the_exact_form(backend):
    """The stripe average and the orbit traps need every iteration's z in FP64:
    a mixed-form request renders them in the exact form (identical outputs),
    supersampled ones included (their adaptive-SS selection: the set boundary,
    and for traps a colour change of more than 3 palette entries per pixel;
    the cases *_ss3 / *_ss13 hold them to the oracle and the reference build)."""
    for name in ("exterior1000_sac", "minibrot875_trap", "c1_sac", "c1_trap_ss3", "shallow_sac_ss3"):
        c = CASES[name]
        it, _, en, _ = gpu_render(backend, c)
        mit, _, men, _ = gpu_render(backend, c, precision_mode=mbx.PRECISION_MIXED)
        assert np.array_equal(it.view(np.uint32), mit.view(np.uint32)) and np.array_equal(en, men), name
