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
from conftest import load_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    be = mbx.create_compute_backend("cuda")
    yield be
    be.close()


# Tolerances the reference's verify harness applies to its own engine against
# each arbitrary-precision golden (verify.cpp:11837-11881, gui case :376):
# class-exact, and (max, mean, p99) of |smooth value difference|.
TRUTH_TOL = {
    "minibrot875": (1.0, None, None),
    "extref875": (1.0, None, None),
    "gui875": (1.0, None, None),
    "slowpoint": (90000.0, 300.0, 3000.0),
    "point31": (12000.0, 200.0, 4000.0),
}


def test_mixed_on_parity_cases(backend):
    """Every perturbation parity case in mixed precision. Cases with the
    reference's arbitrary-precision golden files are held to the tolerances its
    verify harness applies to its engine (TRUTH_TOL); the others to class
    agreement with the exact form and 99.9 % identical escape iterations. DE
    colourings have no FP32 form and must come out identical to the exact form.
    Frames shallower than the reference's floatexp gate (scale 1e6..1e280) run
    the mixed form's rebasing floatexp lanes with one reference, where the exact
    form runs the double path with glitch re-reference passes."""
    from conftest import GOLDEN

    cases = load_cases()
    for name, c in cases.items():
        if len(c["scale"].split(".")[0]) <= 7:  # scale <= 1e6: the shallow path, not perturbation
            continue
        r = {}
        for mode in (mbx.PRECISION_MIXED, mbx.PRECISION_EXACT):
            req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"],
                                     sub=c["sub"], coloring_method=c["coloring_method"], bailout=c["bailout"], precision_mode=mode)
            assert backend.compute_status(req) == mbx.OK, backend.last_error()
            r[mode] = (req.iterations, req.escape_iteration, backend.last_stats.as_dict())
        mi, mn, mst = r[mbx.PRECISION_MIXED]
        ei, en, _ = r[mbx.PRECISION_EXACT]
        if c["coloring_method"] & (2 | 16 | 64):
            assert np.array_equal(mi, ei) and np.array_equal(mn, en), name
            print("\n[mixed vs exact] %s: DE colouring, exact form used" % name)
            continue
        both = (mi > -5) & (ei > -5)
        same = np.mean(mn[both] == en[both])
        cls = int(np.sum((mi[both] < -1.5) != (ei[both] < -1.5)))
        msg = "[mixed vs exact] %s: N identical %.4f, class mismatches %d, fp64 reruns %d of %d" % (name, same, cls, mst["fp64_reruns"], mi.size)
        truth_path = os.path.join(GOLDEN, "truth_%s.f32" % name)
        if os.path.exists(truth_path):
            t = np.fromfile(truth_path, dtype="<f4")
            valid = (t > -5) & (mi > -5)
            ext = valid & (t > -1.5) & (mi > -1.5)
            tcls = int(np.sum((mi[valid] < -1.5) != (t[valid] < -1.5)))
            dd = np.abs(mi[ext].astype(np.float64) - t[ext])
            d = float(np.max(dd, initial=0.0))
            mean = float(dd.mean()) if dd.size else 0.0
            p99 = float(np.sort(dd)[int(np.ceil(0.99 * dd.size)) - 1]) if dd.size else 0.0
            msg += "; vs truth: class mismatches %d, |dmu| max %.4f mean %.4f p99 %.4f" % (tcls, d, mean, p99)
            print("\n" + msg)
            tmax, tmean, tp99 = TRUTH_TOL[name]
            assert tcls == 0, name
            assert d <= tmax, name
            assert tmean is None or mean <= tmean, name
            assert tp99 is None or p99 <= tp99, name
        else:
            print("\n" + msg)
            assert cls <= max(1, mi.size // 1000), name
            assert same >= 0.999, name


@pytest.mark.parametrize("window", [1e8, 1e12, 1e16])
@pytest.mark.parametrize("bps", [3, 4])
def test_every_autotuner_shape_keeps_accuracy(window, bps):
    """The autotuner picks launch shapes and rescale windows by speed alone, so
    each shape it may pick must hold the accuracy bar: the minibrot frames with
    arbitrary-precision goldens (most samples need the rerun tiers) class-exact
    and within the verify harness's |dmu| bound."""
    from conftest import GOLDEN

    cases = load_cases()
    be = mbx.create_compute_backend("cuda")
    try:
        be.set_tuning(256, bps, 0, window)
        for name in ("minibrot875", "extref875", "gui875"):
            c = cases[name]
            out = {}
            for mode in (mbx.PRECISION_MIXED, mbx.PRECISION_EXACT):
                req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"],
                                         sub=c["sub"], coloring_method=c["coloring_method"], bailout=c["bailout"], precision_mode=mode)
                assert be.compute_status(req) == mbx.OK, be.last_error()
                out[mode] = (req.iterations, req.escape_iteration)
            mi, mn = out[mbx.PRECISION_MIXED]
            ei, en = out[mbx.PRECISION_EXACT]
            t = np.fromfile(os.path.join(GOLDEN, "truth_%s.f32" % name), dtype="<f4")
            valid = (t > -5) & (mi > -5)
            ext = valid & (t > -1.5) & (mi > -1.5)
            assert int(np.sum((mi[valid] < -1.5) != (t[valid] < -1.5))) == 0, (name, window, bps)
            assert float(np.max(np.abs(mi[ext].astype(np.float64) - t[ext]), initial=0.0)) <= TRUTH_TOL[name][0], (name, window, bps)
            both = (mi > -5) & (ei > -5)
            print("\n[shape %d bps, window %.0e] %s: N identical to the exact form %.4f" % (bps, window, name, np.mean(mn[both] == en[both])))
    finally:
        be.close()
