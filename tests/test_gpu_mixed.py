"""Mixed-precision (FP32 floatexp) form against arbitrary-precision truth.

The mixed form is not bit-identical to the reference; the bar is the north-star
accuracy statement: on a seeded subset of samples, the fraction whose escape
iteration equals the brute-force arbitrary-precision iteration (the reference's
own per-pixel oracle, accuratePointCompute, at the frame's precision), the class
agreement, and the largest smooth-value error. Figures are printed for the
record (pytest -s) and asserted against the thresholds below.
"""
import os

import numpy as np
import pytest

import mbx
import oracle
import views
from conftest import load_cases

pytestmark = pytest.mark.gpu

W, H = 480, 270
SUBSET = int(os.environ.get("MBX_TRUTH_SUBSET", "512"))


@pytest.fixture(scope="module")
def backend():
    be = mbx.create_compute_backend("cuda")
    yield be
    be.close()


def render(be, v, mode, w=W, h=H):
    req = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], w, h, v["max_iterations"], bailout=v["bailout"], precision_mode=mode)
    assert be.compute_status(req) == mbx.OK, be.last_error()
    return req.iterations, req.escape_iteration, be.last_stats.as_dict()


@pytest.mark.parametrize("k", [300, 1000])
def test_mixed_vs_truth(backend, k):
    v = views.deep_view(k, width=W, height=H)
    mit, men, mst = render(backend, v, mbx.PRECISION_MIXED)
    eit, een, est = render(backend, v, mbx.PRECISION_EXACT)
    rng = np.random.RandomState(4096 + k)
    idx = np.sort(rng.choice(W * H, size=SUBSET, replace=False))
    keys = np.stack([idx // W, idx % W, np.zeros_like(idx), np.zeros_like(idx)], axis=1)
    tv, tn = oracle.truth(v["center_re"], v["center_im"], v["scale"], W, H, v["max_iterations"], keys, bailout=v["bailout"], threads=os.cpu_count())
    m_same = np.mean(men[idx] == tn)
    e_same = np.mean(een[idx] == tn)
    cls = int(np.sum((men[idx] < 0) != (tn < 0)))
    ext = (tn > 0) & (men[idx] > 0)
    maxdmu = float(np.max(np.abs(mit[idx][ext].astype(np.float64) - tv[ext]), initial=0.0))
    full_same = np.mean(men == een)
    print("\n[accuracy] 1e-%d: mixed N==truth %.5f  exact N==truth %.5f  class mismatches %d  max |dmu| %.3g  mixed==exact (full frame) %.5f  subset %d" % (k, m_same, e_same, cls, maxdmu, full_same, SUBSET))
    assert cls == 0
    assert m_same >= 0.999


def test_mixed_on_parity_cases(backend):
    """Floatexp parity cases in mixed precision: against the reference's own
    arbitrary-precision golden files with the tolerances its verify harness
    applies to its engine (verify.cpp:11837-11857), and class-exact against the
    exact form elsewhere."""
    from conftest import GOLDEN

    cases = load_cases()
    for name in ("minibrot875", "extref875", "deep876", "exterior1000", "subpixel737"):
        c = cases[name]
        r = {}
        for mode in (mbx.PRECISION_MIXED, mbx.PRECISION_EXACT):
            req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"], bailout=c["bailout"], precision_mode=mode)
            assert backend.compute_status(req) == mbx.OK, backend.last_error()
            r[mode] = (req.iterations, req.escape_iteration)
        mi, mn = r[mbx.PRECISION_MIXED]
        ei, en = r[mbx.PRECISION_EXACT]
        same = np.mean(mn == en)
        cls = int(np.sum((mn < 0) != (en < 0)))
        msg = "[mixed vs exact] %s: N identical %.4f, class mismatches %d" % (name, same, cls)
        truth_path = os.path.join(GOLDEN, "truth_%s.f32" % name)
        if os.path.exists(truth_path):
            t = np.fromfile(truth_path, dtype="<f4")
            ext = (t > -1.5) & (mi > -1.5)
            tcls = int(np.sum((mi < -1.5) != (t < -1.5)))
            d = float(np.max(np.abs(mi[ext].astype(np.float64) - t[ext]), initial=0.0))
            msg += "; vs truth: class mismatches %d, max |dmu| %.4f" % (tcls, d)
            assert tcls == 0, name
            assert d <= 1.0, name
        print("\n" + msg)
        assert cls == 0, name
