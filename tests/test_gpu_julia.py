"""Julia frames (MBX_MODE_JULIA, Mandel::ComputeJulia mp.cpp:992-1044) on the
GPU against the reference engine's own output (tests/golden/ref_julia_*.f32,
written by the reference's ComputeJulia) and the oracle's restatement.

The kernel runs the reference's double operations in its order without FMA;
only the final log of the smooth value comes from a different libm, so the
class and escape index are exact and the value agrees to 1e-6 relative (in
practice bit for bit, bar a last-ulp log difference that survives rounding to
float).
"""
import numpy as np
import pytest

import mbx
import oracle
from conftest import load_julia_cases, load_julia_fixture

pytestmark = pytest.mark.gpu

CASES = load_julia_cases()


def _req(c, **kw):
    return mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"], coloring_method=c["coloring_method"],
                              bailout=c["bailout"], full_height=c.get("full_height", 0), row_base=c.get("row_base", 0), compute_mode=mbx.MODE_JULIA,
                              fixed_c_re=c["fixed_c_re"], fixed_c_im=c["fixed_c_im"], **kw)


@pytest.fixture(scope="module")
def be():
    b = mbx.create_compute_backend("cuda")
    yield b
    b.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_julia_matches_reference(be, name):
    c = CASES[name]
    req = _req(c)
    assert be.compute_status(req) == mbx.OK, be.last_error()
    ref = load_julia_fixture(name)
    it, en = oracle.julia(c["center_re"], c["center_im"], c["scale"], c["fixed_c_re"], c["fixed_c_im"], c["width"], c["height"], c["max_iterations"], c["coloring_method"], c["bailout"], c.get("full_height", 0), c.get("row_base", 0))
    assert np.array_equal(req.escape_iteration, en)
    assert np.array_equal(req.iterations < -1.5, ref < -1.5)
    np.testing.assert_allclose(req.iterations, ref, rtol=1e-6, atol=0)
    same = float(np.mean(req.iterations.view(np.uint32) == ref.view(np.uint32)))
    assert same > 0.999, same
    st = be.last_stats
    assert st.kernel_launches == 1 and st.samples == c["width"] * c["height"]


def test_julia_strips_match_oracle(be):
    """Strips of a frame (full_height / row_base): each strip is its own
    ComputeJulia with the frame's spacing and an offset corner, so it is checked
    against the oracle's strip, not against rows of the whole frame (their
    corners differ in the last bits)."""
    c = dict(CASES["rabbit"])
    for base in range(0, c["height"], 40):
        s = dict(c, height=min(40, c["height"] - base), full_height=c["height"], row_base=base)
        r = _req(s)
        assert be.compute_status(r) == mbx.OK, be.last_error()
        it, en = oracle.julia(s["center_re"], s["center_im"], s["scale"], s["fixed_c_re"], s["fixed_c_im"], s["width"], s["height"], s["max_iterations"], s["coloring_method"], s["bailout"], s["full_height"], s["row_base"])
        assert np.array_equal(r.escape_iteration, en)
        np.testing.assert_allclose(r.iterations, it, rtol=1e-6, atol=0)


def test_julia_device_outputs(be):
    torch = pytest.importorskip("torch")
    c = CASES["dendrite_ede"]
    n = c["width"] * c["height"]
    dv = torch.empty(n, dtype=torch.float32, device="cuda")
    dn = torch.empty(n, dtype=torch.int32, device="cuda")
    req = _req(c, iterations=dv, escape_iteration=dn)
    assert be.compute_status(req) == mbx.OK, be.last_error()
    host = _req(c)
    assert be.compute_status(host) == mbx.OK
    assert np.array_equal(dv.cpu().numpy(), host.iterations) and np.array_equal(dn.cpu().numpy(), host.escape_iteration)


def test_invalid_julia_requests(be):
    c = CASES["rabbit"]
    for kw in (dict(sub=3), dict(coloring_method=mbx.DE_OVERLAY), dict(fixed_c_re=None)):
        d = dict(c)
        req = _req(d)
        for k, v in kw.items():
            setattr(req, k, v)
        assert be.compute_status(req) == mbx.E_INVALID
    req = _req(c)
    req.compute_mode = 7
    assert be.compute_status(req) == mbx.E_INVALID
    assert be.compute_batch([_req(c)]) == mbx.E_INVALID
