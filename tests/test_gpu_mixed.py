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


def truth_values(name):
    """Arbitrary-precision values of a parity case: the reference's own golden
    file (truth_<name>.f32) or the oracle's full-frame truth
    (truthgen_<name>.npz, tests/golden/make_truth.py --cases); None if neither."""
    from conftest import GOLDEN

    p = os.path.join(GOLDEN, "truth_%s.f32" % name)
    if os.path.exists(p):
        return np.fromfile(p, dtype="<f4")
    p = os.path.join(GOLDEN, "truthgen_%s.npz" % name)
    if os.path.exists(p):
        return np.load(p)["value"]
    return None


def vs_truth(values, t):
    """(class mismatches, fraction of escaping samples within 1 of the truth's
    smooth value, mean, p99 and max |dmu|) of a render against truth values."""
    valid = (t > -5) & (values > -5)
    ext = valid & (t > -1.5) & (values > -1.5)
    cls = int(np.sum((values[valid] < -1.5) != (t[valid] < -1.5)))
    dd = np.abs(values[ext].astype(np.float64) - t[ext])
    if dd.size == 0:
        return cls, 1.0, 0.0, 0.0, 0.0
    return cls, float(np.mean(dd < 1.0)), float(dd.mean()), float(np.sort(dd)[int(np.ceil(0.99 * dd.size)) - 1]), float(dd.max())


def test_mixed_on_parity_cases(backend):
    """Every perturbation parity case in mixed precision.

    * DE colourings: test_mixed_de_colourings.
    * Floatexp frames (scale > 1e280): cases with the reference's
      arbitrary-precision golden files are held to the tolerances its verify
      harness applies to its engine (TRUTH_TOL); the others to class agreement
      with the exact form and 99.9 % identical escape iterations.
    * Frames below the reference's floatexp gate (scale 1e6..1e280) run the
      mixed form's rebasing floatexp lanes with one reference, where the exact
      form runs the reference's double path with glitch re-reference passes; on
      chaotic samples both leave the true orbit, differently. They are held to
      truth (the reference's golden file or the oracle's full-frame truth):
      no more class mismatches than the exact form, at least as many samples
      within 1 of the truth's smooth value (less 0.5 %), a mean |dmu| no worse
      than 1.1 times the exact form's, and TRUTH_TOL where it applies.
    """
    cases = load_cases()
    for name, c in cases.items():
        if len(c["scale"].split(".")[0]) <= 7:  # scale <= 1e6: the shallow path, not perturbation
            continue
        if c["coloring_method"] & (8 | 32):  # orbit colourings take the exact form (test_gpu_parity)
            continue
        r = {}
        for mode in (mbx.PRECISION_MIXED, mbx.PRECISION_EXACT):
            req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"],
                                     sub=c["sub"], coloring_method=c["coloring_method"], bailout=c["bailout"], precision_mode=mode)
            assert backend.compute_status(req) == mbx.OK, backend.last_error()
            r[mode] = (req.iterations, req.escape_iteration, backend.last_stats.as_dict())
        mi, mn, mst = r[mbx.PRECISION_MIXED]
        ei, en, est = r[mbx.PRECISION_EXACT]
        if c["coloring_method"] & (2 | 16 | 64):
            continue  # test_mixed_de_colourings
        both = (mi > -5) & (ei > -5)
        same = np.mean(mn[both] == en[both])
        cls = int(np.sum((mi[both] < -1.5) != (ei[both] < -1.5)))
        msg = "[mixed vs exact] %s: N identical %.4f, class mismatches %d, fp64 reruns %d of %d" % (name, same, cls, mst["fp64_reruns"], mi.size)
        t = truth_values(name)
        double_path = not est["used_floatexp"]
        if t is not None:
            mc, mfrac, mmean, mp99, mmax = vs_truth(mi, t)
            ec, efrac, emean, ep99, emax = vs_truth(ei, t)
            msg += "; vs truth: mixed class %d, within 1: %.4f, |dmu| mean %.3f p99 %.3f max %.3f; exact class %d, within 1: %.4f, mean %.3f p99 %.3f max %.3f" % (
                mc, mfrac, mmean, mp99, mmax, ec, efrac, emean, ep99, emax)
            print("\n" + msg)
            if name in TRUTH_TOL:
                tmax, tmean, tp99 = TRUTH_TOL[name]
                assert mc == 0, name
                assert mmax <= tmax, name
                assert tmean is None or mmean <= tmean, name
                assert tp99 is None or mp99 <= tp99, name
            if double_path:
                assert mst["used_floatexp"] == 1, name
                assert mc <= ec, name
                assert mfrac >= efrac - 0.005, name
                assert mmean <= 1.1 * emean + 1e-3, name
            elif name not in TRUTH_TOL:
                assert cls <= max(1, mi.size // 1000), name
                assert same >= 0.999, name
        else:
            print("\n" + msg)
            assert not double_path, "%s: a double-path case needs truth (tests/golden/make_truth.py --cases)" % name
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


# The DE value of a sample is |z| log|z|^2 / (dx |dz/dc|); in the mixed form the
# derivative is carried in the lane type (FP32 floatexp in the FP32 tier) and the
# value formed in FP64 floatexp. Bars against arbitrary-precision truth (the
# oracle's GMP orbit and derivative, tests/golden/truthgen_<case>.npz), over the
# samples whose N equals the truth's:
DE_REL_P999 = 1e-4   # 99.9th percentile of |dDE| / DE
DE_REL_MAX = 1e-3    # largest |dDE| / DE
ANGLE_P999 = 1e-4    # normal map: 99.9th percentile of |d angle| (radians, mod 2 pi)
ANGLE_MAX = 1e-3


def test_lane_budget_changes_no_result():
    """The autotuner's lane-span axis (iterations a lane walks per call between
    its warp's refill points) changes only where calls end: the outputs of a
    frame whose samples take every tier, with and without interior detection
    and with the derivative, are bit-identical at 64, 256 and 1024."""
    cases = load_cases()
    be = mbx.create_compute_backend("cuda")
    try:
        for name, cm in (("minibrot875", None), ("subpixel737", None), ("minibrot875", 1)):
            c = cases[name]
            ref = None
            for lb in (256, 64, 1024):
                be.set_lane_budget(lb)
                req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"], sub=c["sub"],
                                         coloring_method=c["coloring_method"] if cm is None else cm, bailout=c["bailout"],
                                         precision_mode=mbx.PRECISION_MIXED)
                assert be.compute_status(req) == mbx.OK, be.last_error()
                out = (req.iterations.copy(), req.escape_iteration.copy())
                if ref is None:
                    ref = out
                else:
                    assert np.array_equal(out[0], ref[0]) and np.array_equal(out[1], ref[1]), (name, cm, lb)
    finally:
        be.close()


def _de_errors(values, n, tv, tn, angle, skip=None):
    ok = (n == tn) & (tn > 0) & (values > -5)
    if skip is not None:
        ok &= ~skip
    if angle:
        d = np.abs(np.angle(np.exp(1j * (values[ok].astype(np.float64) - tv[ok].astype(np.float64)))))
    else:
        a, b = values[ok].astype(np.float64), tv[ok].astype(np.float64)
        d = np.where(b == 0, np.abs(a), np.abs(a - b) / np.maximum(np.abs(b), 1e-300))
    if d.size == 0:
        return 0.0, 0.0, 0
    return float(np.sort(d)[int(np.ceil(0.999 * d.size)) - 1]), float(d.max()), int(d.size)


def test_mixed_de_colourings(backend):
    """Every perturbation parity case with a DE colouring (EDE, DE overlay,
    normal map) in mixed precision against arbitrary-precision truth: class
    agreement, 99.9 % of the escape iterations equal to the truth's, and the
    distance (or the normal-map angle) within the stated bounds on the samples
    whose N agree, or no worse than the exact form where the exact form itself
    misses them (samples no lane tier can vouch for finish in the exact form).
    The exact form's distances to the same truth are printed beside them: on
    minibrot875 the reference's FP64 derivative is off by up to 14 % on a few
    samples where the mixed form's lanes are within 1e-7."""
    from conftest import GOLDEN

    cases = load_cases()
    seen = 0
    for name, c in cases.items():
        if len(c["scale"].split(".")[0]) <= 7 or not (c["coloring_method"] & (2 | 16 | 64)):
            continue
        tp = os.path.join(GOLDEN, "truthgen_%s.npz" % name)
        assert os.path.exists(tp), "%s: no truth (tests/golden/make_truth.py --cases %s)" % (name, name)
        z = np.load(tp)
        tv, tn = z["value"], z["N"]
        r = {}
        for mode in (mbx.PRECISION_MIXED, mbx.PRECISION_EXACT):
            req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"],
                                     sub=c["sub"], coloring_method=c["coloring_method"], bailout=c["bailout"], precision_mode=mode)
            assert backend.compute_status(req) == mbx.OK, backend.last_error()
            r[mode] = (req.iterations.copy(), None if req.normal is None else req.normal.copy(), req.escape_iteration.copy(), backend.last_stats.as_dict())
        mi, mnr, mn, mst = r[mbx.PRECISION_MIXED]
        ei, enr, en, _ = r[mbx.PRECISION_EXACT]
        assert mst["fp32_pass_steps"] > 0, name + ": the mixed form did not run its FP32 lanes"
        valid = (mi > -5) & (tn != -10)
        cls = int(np.sum((mn[valid] < 0) != (tn[valid] < 0)))
        same_n = float(np.mean(mn[valid] == tn[valid]))
        cm = c["coloring_method"]
        angle = bool(cm & 16) and not (cm & 2)
        if cm & 2:
            mv, ev = mi, ei
        else:
            mv, ev = mnr, enr
        # samples whose distance / angle both forms leave at 0: the reference
        # pixel (its value comes from the reference orbit) and, under adaptive
        # supersampling, the sub-samples of pixels that were not flagged
        refpix = None
        if not (cm & 2):
            refpix = (mv == 0) & (ev == 0) & (tv != 0) & (tn > 0)
            assert c["sub"] > 1 or refpix.sum() <= 1, name
        mp, mmax, cnt = _de_errors(mv, mn, tv, tn, angle, refpix)
        ep, emax, _ = _de_errors(ev, en, tv, tn, angle, refpix)
        what = "angle |d|" if angle else "|dDE|/DE"
        print("\n[mixed DE vs truth] %s: N identical %.5f, class mismatches %d, %s p99.9 %.3g max %.3g over %d samples (exact form: p99.9 %.3g max %.3g); reruns %d of %d"
              % (name, same_n, cls, what, mp, mmax, cnt, ep, emax, mst["fp64_reruns"], mi.size))
        assert cls == 0, name
        assert same_n >= 0.999, name
        # within the bounds, or no worse than the exact form where the exact
        # form itself misses them (its samples are the mixed form's last tier)
        assert mp <= max(ANGLE_P999 if angle else DE_REL_P999, ep), name
        assert mmax <= max(ANGLE_MAX if angle else DE_REL_MAX, emax), name
        seen += 1
    assert seen >= 7
