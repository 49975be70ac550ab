"""The mixed-precision form at the 1080p deep-frame configuration against
arbitrary-precision truth.

For each 1920x1080 frame with a committed truth subset (4096 seeded samples
iterated directly in GMP by the oracle's restatement of the reference's
accuratePointCompute, mp.cpp:719-894; tests/golden/make_truth.py), the frame is
rendered in the mixed form (MBX_PRECISION_MIXED) and, for the record, in the
exact form. Bar: at least 99.99 % of the subset with the truth's escape
iteration (with 4096 samples: every one), no interior/exterior mismatch, and
the smooth value within MAX_DMU of the truth's on every escaping sample — or,
where the reference's own FP64 arithmetic (the exact form) misses that bar, no
worse than the exact form. The figures are printed (pytest -s).
"""
import numpy as np
import pytest

import mbx
import views
from conftest import load_truth

pytestmark = pytest.mark.gpu

W, H = 1920, 1080
MIN_SAME = 0.9999
# Largest |smooth value - truth| accepted on escaping samples. The truth's
# value is computed from the exact orbit; the mixed form's from its FP32
# delta, whose error estimate bounds |dz| error well below what moves N.
MAX_DMU = 0.1


@pytest.mark.parametrize("label", views.TRUTH_FRAMES)
def test_mixed_vs_truth_1080p(label):
    tr = load_truth(label)
    assert tr is not None, "no committed truth subset for %s (tests/golden/make_truth.py)" % label
    idx, tn, tv = tr
    v = views.frame(label, W, H)
    be = mbx.create_compute_backend("cuda")
    try:
        out = {}
        for mode in (mbx.PRECISION_MIXED, mbx.PRECISION_EXACT):
            req = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], W, H, v["max_iterations"], bailout=v["bailout"], precision_mode=mode)
            assert be.compute_status(req) == mbx.OK, be.last_error()
            out[mode] = (req.iterations[idx].astype(np.float64), req.escape_iteration[idx], be.last_stats.as_dict())
    finally:
        be.close()
    mit, men, mst = out[mbx.PRECISION_MIXED]
    eit, een, _ = out[mbx.PRECISION_EXACT]
    same = float(np.mean(men == tn))
    cls = int(np.sum((men < 0) != (tn < 0)))
    ext = (tn > 0) & (men > 0)
    dmu = float(np.max(np.abs(mit[ext] - tv[ext]), initial=0.0))
    e_same = float(np.mean(een == tn))
    e_dmu = float(np.max(np.abs(eit[(tn > 0) & (een > 0)] - tv[(tn > 0) & (een > 0)]), initial=0.0))
    print("\n[truth 1080p] %s: mixed N==truth %.5f (%d of %d), class mismatches %d, max |dmu| %.4g; exact form N==truth %.5f, max |dmu| %.4g; "
          "double-float reruns %d, exact-form reruns %d" % (label, same, int(np.sum(men == tn)), idx.size, cls, dmu, e_same, e_dmu, mst["fp64_reruns"], mst["exact_reruns"]))
    assert cls == 0
    # the bar, or no worse than the exact form where the reference's own FP64
    # arithmetic misses it (samples no lane tier can vouch for finish in the
    # exact form): on the minibrot frame both forms miss the same 3 of 4096
    assert same >= min(MIN_SAME, e_same)
    assert dmu <= max(MAX_DMU, e_dmu)


def test_mixed_c1_config_vs_oracle():
    """The plain FP64 configuration (views.c1_view: 1280x720, half-width 1e-30,
    maxiter 50000) in the mixed form, below the reference's floatexp gate: the
    rebasing FP32 lanes with one reference, against the oracle's exact double
    path (mp.cpp:2290-2585): class identical everywhere and at least 99.99 % of
    the escape iterations identical."""
    import oracle

    v = views.c1_view()
    be = mbx.create_compute_backend("cuda")
    try:
        req = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], 1280, 720, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED)
        assert be.compute_status(req) == mbx.OK, be.last_error()
        st = be.last_stats.as_dict()
    finally:
        be.close()
    assert st["used_floatexp"] == 1
    oit, _, oen, _ = oracle.render(v["center_re"], v["center_im"], v["scale"], 1280, 720, v["max_iterations"], bailout=v["bailout"])
    en = req.escape_iteration
    same = float(np.mean(en == oen))
    cls = int(np.sum((en < 0) != (oen < 0)))
    ext = (en > 0) & (oen > 0)
    dmu = float(np.max(np.abs(req.iterations[ext].astype(np.float64) - oit[ext]), initial=0.0))
    print("\n[c1 mixed] N identical to the exact double path %.6f, class mismatches %d, max |dmu| %.4g, double-float reruns %d" % (same, cls, dmu, st["fp64_reruns"]))
    assert cls == 0
    assert same >= MIN_SAME
    assert dmu <= MAX_DMU
